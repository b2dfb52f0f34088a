"""The bench's multi-rank path on the CPU (gloo, world size 2).

The verified product does not shard: `bench.py --gpus N` runs N independent
replicas, one per rank, with a barrier on both sides of the timed region and
the step time taken as the maximum over ranks.  These tests run that host
logic as two gloo ranks on 127.0.0.1: the barrier and max-over-ranks helpers,
and the reference arm launched the way a multi-GPU run launches it, where
rank 0 alone times the CPU product and prints the one JSON line.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        # rank r reports a step time of 1.5 + r ms: every rank must see the max
        got = bench.max_over_ranks(1.5 + rank, world)
        bench.barrier(world)
        Path(out_dir, f"rank{rank}.txt").write_text(repr(got))
    finally:
        dist.destroy_process_group()


def test_barrier_and_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    for r in range(world):
        assert float(Path(tmp_path, f"rank{r}.txt").read_text()) == 2.5


def test_single_rank_helpers_need_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    bench.barrier(1)
    assert bench.max_over_ranks(3.25, 1) == 3.25


def test_reference_arm_under_torchrun_prints_one_line_from_rank0():
    """`bench.py --impl reference` launched on two ranks: the CPU product is
    timed by rank 0 only (a small row panel here), the other rank exits 0
    without work, and stdout carries exactly one JSON line."""
    oracle_build = pytest.importorskip("oracle.build")
    oracle_build.build_oracle()
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--size", "128", "--cpu-rows", "8"]
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["steps"] == 1
    assert rec["value"] > 0 and rec["e2e"]["value"] == rec["value"]
    assert rec["cpu_baseline"]["kind"] == "port"
    # the keys of the one-line contract both arms print
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert key in rec, key
    assert rec["higher_is_better"] is True and rec["scaling"] == "weak"
    assert rec["e2e"]["h2d_bytes_per_step"] == 0 and rec["e2e"]["d2h_bytes_per_step"] == 0
    assert rec["config"]["workload"] and rec["config"]["n"] == 128
    assert rec["cpu_baseline"]["cores"] >= 1 and rec["cpu_baseline"]["value"] == rec["value"]
