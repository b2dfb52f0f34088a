"""Benchmark: verified interval GEMM at n = 8192 on one GB300 (per rank).

Workload ("interval GEMM n=8192"): C = [A] * [B] with A, B square n x n
interval matrices in kv layout; midpoints have mantissa uniform in [1, 2),
random sign and exponent uniform in [-4, 4]; radius = 2^-40 |mid| (seeded,
synthetic).  Throughput is 2 n^3 / t (one real GEMM's worth per product).

Our arm (default) prints one JSON line with
  value          TFLOP/s of the headline form, inputs resident in HBM, CUDA
                 events on the launching stream over exactly --steps calls;
  e2e            the same metric through the host-pointer C ABI call
                 (vcpcu_igemm) from pinned host buffers: H2D of A and B and
                 D2H of C inside the timed region, every step;
  plain          the plain FP64 __fma_rd/__fma_ru form on the same inputs
                 (its own TFLOP/s), and the enclosure-width comparison;
  roofline       the dominant kernel against the measured peak;
  cpu_baseline   the CPU restatement of pidblas::mulmm (oracle port of the
                 reference path) on the host cores, bounded row sample.
--impl reference times that CPU path alone as the reference arm.

Inputs are 1 GiB per operand (larger than the 129 MB L2), so no L2 flush is
needed between steps.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "verified interval GEMM TFLOP/s n=8192: Ozaki-TC vs FP64 RU/RD, equal width"
UNIT = "TFLOP/s"
WORKLOAD = "interval GEMM n=8192, mid E(phi=4), rad 2^-40|mid|"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--form", default="auto", choices=["auto", "plain", "ozaki"])
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-rows", type=int, default=0, help="row sample of the CPU baseline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only-headline", action="store_true",
                    help="time the headline form only (profiling runs): no plain form, "
                         "width, containment, e2e or CPU legs")
    return ap.parse_args()


# ---------------------------------------------------------------- dist setup
def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int, device=None) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during timing."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- helpers
def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def make_inputs(n: int, seed: int):
    from vcp_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    A = W.interval_ephi(rng, n, n, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, n, n, 4, 2.0 ** -40)
    return A, B


def cpu_baseline(A, B, n, rows, threads):
    """oracle port of pidblas::mulmm on a row panel (rows x n times n x n)."""
    from oracle import oracle as O
    Ap = A.reshape(n, n, 2)[:, :rows, :].copy().reshape(-1)  # first `rows` rows, all k
    t0 = time.perf_counter()
    O.pidblas_mulmm(rows, n, n, Ap, B, threads)
    dt = time.perf_counter() - t0
    return 2.0 * rows * n * n / dt / 1e12, dt


def cpu_count():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---------------------------------------------------------------- reference arm
def run_reference(args, ws, rank):
    if rank != 0:
        return
    n = args.n
    A, B = make_inputs(n, 1234)
    threads = cpu_count()
    rows = args.cpu_rows or 128
    for _ in range(max(args.warmup, 0) and 1):
        cpu_baseline(A, B, n, 16, threads)
    vals, times = [], []
    for _ in range(args.steps):
        v, dt = cpu_baseline(A, B, n, rows, threads)
        vals.append(v)
        times.append(dt)
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * 2.0 * n ** 3 / (v * 1e12),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "n": n, "form": "pidblas (CPU)",
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{rows} x {n} x {n} row panel per step "
                                   f"(~{statistics.median(times):.1f} s), oracle restatement of "
                                   "pidblas::mulmm over the vblas sequential-chain dgemm"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm
def run_ours(args, ws, rank, local):
    import torch
    from vcp_gb300 import _lib, pidcuda
    from vcp_gb300.build import build

    if rank == 0:
        build()
    barrier(ws)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load()
    n = args.n
    A, B = make_inputs(n, 1234 + rank)
    dA = torch.from_numpy(A).to(dev)
    dB = torch.from_numpy(B).to(dev)
    dC = torch.empty(2 * n * n, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)

    have_ozaki = True
    try:
        with torch.cuda.stream(stream):
            pidcuda.mulmm_dev(64, 64, 64, dA, n, dB, n, dC, 64, pidcuda.FORM_OZAKI, 0, stream)
        stream.synchronize()
    except Exception:
        have_ozaki = False
    form_name = args.form
    if form_name == "auto":
        form_name = "ozaki" if have_ozaki else "plain"
    form = pidcuda.FORM_OZAKI if form_name == "ozaki" else pidcuda.FORM_PLAIN

    def one(f, slices=args.slices):
        pidcuda.mulmm_dev(n, n, n, dA, n, dB, n, dC, n, f, slices, stream)

    def timed(f, steps, warmup):
        for _ in range(warmup):
            one(f)
        stream.synchronize()
        barrier(ws)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = _lib.launch_count()
        e0.record(stream)
        for _ in range(steps):
            one(f)
        e1.record(stream)
        stream.synchronize()
        l1 = _lib.launch_count()
        torch.cuda.synchronize()
        barrier(ws)
        return e0.elapsed_time(e1) / steps, l1 - l0

    if form == pidcuda.FORM_OZAKI:
        _lib.profile(True)
        _lib.profile_read()  # discard anything recorded before the timed region
    with ClockSampler(local) as clk:
        ms, launches = timed(form, args.steps, args.warmup)
    phases, tc_flops = ([0.0] * 4, 0)
    if form == pidcuda.FORM_OZAKI:
        phases, tc_flops = _lib.profile_read()
        _lib.profile(False)
        # the warm-up calls were recorded too: keep the timed steps' share
        frac = args.steps / (args.steps + args.warmup)
        phases = [p * frac for p in phases]
        tc_flops = int(tc_flops * frac)
    ms_max = max_over_ranks(ms, ws, dev)
    value = ws * 2.0 * n ** 3 / (ms_max * 1e-3) / 1e12
    if args.only_headline:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": ws * 2.0 * n ** 3 / (ms_max * 1e-3) / 1e12,
                              "unit": UNIT, "ms_per_step": ms_max, "form": form_name, "n": n,
                              "only_headline": True}), flush=True)
        return
    C_head = dC.cpu().numpy().copy()

    # plain FP64 form on the same inputs (also the width reference)
    if form == pidcuda.FORM_PLAIN:
        plain_ms, C_plain = ms, C_head
    else:
        plain_ms, _ = timed(pidcuda.FORM_PLAIN, args.plain_steps, 1)
        C_plain = dC.cpu().numpy().copy()
    plain_tflops = 2.0 * n ** 3 / (max_over_ranks(plain_ms, ws, dev) * 1e-3) / 1e12

    wh = C_head[1::2] - C_head[0::2]
    wp = C_plain[1::2] - C_plain[0::2]
    width = {"ratio_median": float(np.median(wh / wp)), "ratio_max": float(np.max(wh / wp)),
             "frac_not_wider": float(np.mean(wh <= wp))}

    # containment of the headline result on a seeded sample (exact hull oracle)
    from oracle import oracle as O
    rs = np.random.default_rng(99)
    rows = rs.integers(0, n, 1024)
    cols = rs.integers(0, n, 1024)
    lo, up = O.exact_hull(n, n, n, A, B, rows, cols)
    idx = 2 * (rows + cols * n)
    fails = int(np.sum(C_head[idx] > lo) + np.sum(C_head[idx + 1] < up))

    # e2e through the host-pointer C ABI from pinned buffers
    hA = torch.from_numpy(A).pin_memory()
    hB = torch.from_numpy(B).pin_memory()
    hC = torch.empty(2 * n * n, dtype=torch.float64).pin_memory()
    pa, pb, pc = hA.data_ptr(), hB.data_ptr(), hC.data_ptr()
    e2e_steps = max(1, min(args.steps, 3 if form == pidcuda.FORM_PLAIN else args.steps))
    _lib.call("vcpcu_igemm", n, n, n, pa, pb, pc, form, args.slices)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        _lib.call("vcpcu_igemm", n, n, n, pa, pb, pc, form, args.slices)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    t_e2e = max_over_ranks(t_e2e, ws, dev)
    e2e_val = ws * 2.0 * n ** 3 / t_e2e / 1e12

    # roofline of the dominant kernel
    pk, pk_kind = peaks()
    if form == pidcuda.FORM_PLAIN:
        fp64_peak, fp64_kind = measure_fp64_peak(dev)
        achieved = 8.0 * n ** 3 / (ms * 1e-3) / 1e12
        roof = {"bound": "fp64", "kernel": "interval_gemm_kernel", "achieved": achieved,
                "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                "traffic": None, "peak_kind": fp64_kind,
                "algorithmic": "8 n^3 FP64 flops per launch (4 directed FMA chains)"}
    else:
        roof = ozaki_roofline(phases, tc_flops, args.steps, pk, pk_kind)

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = cpu_count()
        rows_s = args.cpu_rows or 128
        v, dt = cpu_baseline(A, B, n, rows_s, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{rows_s} x {n} x {n} row panel ({dt:.1f} s), oracle restatement of "
                         "pidblas::mulmm over the vblas sequential-chain dgemm"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if form_name == "plain" else "bf16-slices/f64",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "n": n, "form": form_name,
                       "slices": args.slices or "default", "parallelism": f"replicas x{ws}",
                       "l2": "inputs (1 GiB per operand) larger than L2; no flush"},
            "plain": {"value": plain_tflops, "ms_per_step": plain_ms, "steps": args.plain_steps},
            "speedup_vs_plain": value / plain_tflops,
            "width_vs_plain": width,
            "containment_failures": fails, "containment_sample": 1024,
            "e2e": {"value": e2e_val, "unit": UNIT,
                    "h2d_bytes_per_step": int(hA.numel() * 8 + hB.numel() * 8),
                    "d2h_bytes_per_step": int(hC.numel() * 8)},
            "gpu_launches": int(launches),
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)


def measure_fp64_peak(dev):
    """cuBLAS DGEMM throughput at 8192^3 (a library GEMM, best of 3)."""
    import torch
    try:
        a = torch.randn(8192, 8192, dtype=torch.float64, device=dev)
        b = torch.randn(8192, 8192, dtype=torch.float64, device=dev)
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        return 2.0 * 8192 ** 3 / (best * 1e-3) / 1e12, "measured (cuBLAS DGEMM 8192^3)"
    except Exception:
        return 1.25, "nominal"


def ozaki_roofline(phases, tc_flops, steps, pk, pk_kind):
    """Dominant kernel oz_slice_gemm_kernel (three launches per call): the
    algorithmic bf16 tensor flops (2 m n k per slice pair) over their summed
    CUDA-event time on the launching stream."""
    gemm_ms = sum(phases[1:4])
    achieved = tc_flops / (gemm_ms * 1e-3) / 1e12 if gemm_ms > 0 else None
    peak = pk.get("bf16_tflops", 1900.0)
    return {"bound": "tensor", "kernel": "oz_slice_gemm_kernel", "achieved": achieved,
            "peak": peak, "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
            "traffic": None, "peak_kind": f"{pk_kind} bf16 dense (burst)",
            "algorithmic": "2*m*n*k per bf16 slice-pair product",
            "phase_ms_per_call": {"prep": phases[0] / steps, "radius1": phases[1] / steps,
                                  "radius2": phases[2] / steps, "midpoint": phases[3] / steps}}


def main():
    args = parse()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
