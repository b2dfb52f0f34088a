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
  also           short runs of the other benchmark workloads in the same
                 process (``--workload`` runs one of them at full size):
                 cfg1   the n = 512 interval product: CPU port of pidblas vs
                        the GPU's plain form (bits compared) and Ozaki form;
                 batch  4096 uneven interval GEMMs, m, n, k log-uniform in
                        [32, 1024], mid U[-1, 1], rad 1e-12 |mid|: throughput
                        and p50 / p99 per-problem latency from device stamps,
                        plain vs Ozaki vs AUTO, each a captured CUDA graph;
                 dd     dd GEMM (pddblas semantics), hi E(phi), lo = hi 2^-53 u:
                        TFLOP/s, relative error against the exact product and
                        the tightness of the returned bound;
                 point  up/down point GEMM (udmatmul shape), entries E(phi):
                        plain RU/RD FMA chains vs the Ozaki enclosure at
                        slice counts s, width ratio and containment;
                 lss    the verification of imats::linearsolve on the GPU
                        (vcpcu_ilss_verify), n x n with nrhs right-hand
                        sides (--phis carries nrhs): plain vs Ozaki time,
                        width ratio, CPU restatement;
                 eig    the verification of imats::eigsymge on the GPU
                        (vcpcu_ieigsymge stages), n x n: plain vs Ozaki;
                 emden  the verified solution of -Laplace u = u^2 on the
                        unit square (test_PDE/test_Emden.cpp), Legendre
                        orders M (--sizes, default 30, 50, 70): Newton, the
                        inverse-norm, residual and Kantorovich bounds, plain
                        vs Ozaki vs the CPU pipeline; wall time per stage
                        and the verified H^1_0 error bound.
--impl reference times that CPU path alone as the reference arm.

Inputs are 1 GiB per operand (larger than the 129 MB L2), so no L2 flush is
needed between steps.
"""
from __future__ import annotations

import argparse
import gc
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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # --size is the spelling to use under torchrun, whose own parser reads
    # "--n" as an ambiguous abbreviation of its options
    ap.add_argument("--n", "--size", dest="n", type=int, default=8192)
    ap.add_argument("--form", default="auto", choices=["auto", "plain", "ozaki"])
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-rows", type=int, default=0, help="row sample of the CPU baseline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="interval",
                    choices=["interval", "batch", "dd", "point", "lss", "eig", "emden"],
                    help="interval: the headline line (default); the others print their own "
                         "line at the full sizes of that workload")
    ap.add_argument("--sizes", default="", help="point / dd: comma-separated n (or m:n:k)")
    ap.add_argument("--phis", default="", help="point / dd: comma-separated phi")
    ap.add_argument("--slice-list", default="", help="point: comma-separated slice counts")
    ap.add_argument("--no-also", action="store_true", help="skip the short other workloads")
    ap.add_argument("--batch-count", type=int, default=4096,
                    help="batch: number of problems (--form ozaki: the tensor-core form only)")
    ap.add_argument("--no-model-check", action="store_true",
                    help="skip the bit-for-bit host-model check of sampled rows and columns")
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
    """nvidia-smi clocks/throttle reasons sampled every 100 ms during timing.
    The sampler is started, and its first (idle) sample read and dropped,
    before the timed region begins, so that every kept sample falls inside
    it."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        import select
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            ready, _, _ = select.select([self.proc.stdout], [], [], 5.0)
            if ready:
                self.proc.stdout.readline()  # the sample before the timed region
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


def headline_config(n: int, ws: int) -> dict:
    """The workload description both arms print (identical for the ratio)."""
    return {"workload": WORKLOAD, "n": n, "parallelism": f"replicas x{ws}",
            "l2": "inputs (1 GiB per operand) larger than L2; no flush"}


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


def model_bitexact_sample(O, A, B, C, n, slices, nrows=8, ncols=8, seed=17):
    """Compare `nrows` full rows and `ncols` full columns of the n x n
    tensor-core product C with the host model run on those rows of A (all of
    B) and on all of A against those columns of B."""
    rs = np.random.default_rng(seed)
    R = np.sort(rs.choice(n, nrows, replace=False))
    Cc = np.sort(rs.choice(n, ncols, replace=False))
    t0 = time.perf_counter()
    Ar = np.ascontiguousarray(A.reshape(n, n, 2)[:, R, :]).ravel()
    ref_r, st1 = O.ozaki_igemm(nrows, n, n, Ar, B, slices, 2, crt=True)
    got_r = np.ascontiguousarray(C.reshape(n, n, 2)[:, R, :]).ravel()
    Bc = np.ascontiguousarray(B.reshape(n, n, 2)[Cc]).ravel()
    ref_c, st2 = O.ozaki_igemm(n, ncols, n, A, Bc, slices, 2, crt=True)
    got_c = np.ascontiguousarray(C.reshape(n, n, 2)[Cc]).ravel()
    mism = int(np.sum(got_r.view(np.int64) != ref_r.view(np.int64)) +
               np.sum(got_c.view(np.int64) != ref_c.view(np.int64)))
    return {"entries": int((nrows + ncols) * n), "rows": int(nrows), "columns": int(ncols),
            "mismatched_words": mism, "model_status": int(st1 | st2),
            "seconds": time.perf_counter() - t0}


def host_fp64_peak_gflops(cores: int):
    """FP64 peak of `cores` host threads, measured: independent fused
    multiply-add chains on every thread (the oracle's probe) for 0.5 s."""
    try:
        from oracle import oracle as O
        return {"gflops": O.fp64_peak_gflops(0.5, cores), "how": "measured: 16 independent "
                "FMA chains per thread (NEON 2-lane on aarch64), 0.5 s"}
    except Exception:
        return None


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
    pk = host_fp64_peak_gflops(threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        # what was timed: one row panel of the product per step
        "ms_per_step": 1e3 * statistics.median(times),
        "step": f"{rows} x {n} x {n} row panel of the n = {n} product "
                f"(value = 2 * {rows} * {n}^2 flops / panel time)",
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "form": "pidblas (CPU port)",
        "config": headline_config(n, args.gpus),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{rows} x {n} x {n} row panel per step "
                                   f"(~{statistics.median(times):.1f} s), oracle restatement of "
                                   "pidblas::mulmm over the vblas sequential-chain dgemm "
                                   "(NEON micro-kernel on aarch64)",
                         "fp64_gflops": 4e3 * v, "host_fp64_peak": pk,
                         "frac_of_host_fp64_peak": (4e3 * v / pk["gflops"]) if pk else None},
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
    # slice count of the tensor-core form: --slices, else the autotuner's
    # pick for these operands (vcpcu_autotune_pick, made once before the
    # timed region as a caller would; it may add the fast radius products)
    slices, slices_src = args.slices, "--slices" if args.slices else "default"
    if form == pidcuda.FORM_OZAKI and not args.slices:
        f0, s0 = pidcuda.autotune_pick(dA, dB, n, n, n, stream)
        if f0 == pidcuda.FORM_OZAKI and s0:
            slices, slices_src = s0, "autotune_pick"

    def one(f):
        pidcuda.mulmm_dev(n, n, n, dA, n, dB, n, dC, n, f, slices if f == form else 0, stream)

    def timed(f, steps, warmup):
        for _ in range(warmup):
            one(f)
        stream.synchronize()
        barrier(ws)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = _lib.launch_count()
        gc.disable()  # no collector pause while the steps are enqueued
        try:
            e0.record(stream)
            for _ in range(steps):
                one(f)
            e1.record(stream)
        finally:
            gc.enable()
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
    phases, tc_flops = ([0.0] * 5, 0)
    if form == pidcuda.FORM_OZAKI:
        phases, tc_flops = _lib.profile_read(5)
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
                              "slices": slices, "slices_source": slices_src,
                              "only_headline": True}), flush=True)
        return
    C_head = dC.cpu().numpy().copy()

    # e2e through the host-pointer C ABI from pinned buffers, right after the
    # device-resident steps (the same warm GPU), clocks sampled over it
    hA = torch.from_numpy(A).pin_memory()
    hB = torch.from_numpy(B).pin_memory()
    hC = torch.empty(2 * n * n, dtype=torch.float64).pin_memory()
    pa, pb, pc = hA.data_ptr(), hB.data_ptr(), hC.data_ptr()
    e2e_steps = max(1, min(args.steps, 3 if form == pidcuda.FORM_PLAIN else args.steps))
    for _ in range(max(1, min(args.warmup, 3))):
        _lib.call("vcpcu_igemm", n, n, n, pa, pb, pc, form, slices)
    barrier(ws)
    with ClockSampler(local) as clk_e2e:
        gc.disable()  # no collector pause inside the timed calls (as timeit does)
        try:
            t0 = time.perf_counter()
            e2e_marks = [t0]
            for _ in range(e2e_steps):
                _lib.call("vcpcu_igemm", n, n, n, pa, pb, pc, form, slices)
                e2e_marks.append(time.perf_counter())  # the call returns synchronised
            t_e2e = (time.perf_counter() - t0) / e2e_steps
        finally:
            gc.enable()
    e2e_step_ms = [1e3 * (b - a) for a, b in zip(e2e_marks, e2e_marks[1:])]
    t_e2e = max_over_ranks(t_e2e, ws, dev)
    e2e_val = ws * 2.0 * n ** 3 / t_e2e / 1e12
    e2e_h2d, e2e_d2h = int(hA.numel() * 8 + hB.numel() * 8), int(hC.numel() * 8)
    del hA, hB, hC


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

    # bit-for-bit check of sampled full rows and columns of the headline
    # result against the host model of the tensor-core form (each entry
    # depends only on its row of A, its column of B and k)
    model = None
    if form == pidcuda.FORM_OZAKI and rank == 0 and not args.no_model_check:
        model = model_bitexact_sample(O, A, B, C_head, n, slices or 8)

    # the autotuner's pick (form, slice count) for the headline operands and
    # for square 2048 products at exponent spreads 0, 8, 32
    auto_pick = None
    if rank == 0:
        from vcp_gb300 import workloads as W
        f0, s0 = pidcuda.autotune_pick(dA, dB, n, n, n, stream)
        auto_pick = {"headline": {"form": "ozaki" if f0 == pidcuda.FORM_OZAKI else "plain",
                                  "slices": s0}}
        for phi in (0, 8, 32):
            rg = np.random.default_rng(phi)
            Ap = W.interval_ephi(rg, 2048, 2048, phi, 2.0 ** -40)
            Bp = W.interval_ephi(rg, 2048, 2048, phi, 2.0 ** -40)
            f1, s1 = pidcuda.autotune_pick(Ap, Bp, 2048, 2048, 2048)
            auto_pick[f"n2048_phi{phi}_rad2^-40"] = {
                "form": "ozaki" if f1 == pidcuda.FORM_OZAKI else "plain", "slices": s1}

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
        roof = ozaki_roofline(phases, tc_flops, args.steps, pk, pk_kind, n,
                              slices == 8 | pidcuda.SLICES_FAST_RADIUS)

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = cpu_count()
        rows_s = args.cpu_rows
        if not rows_s:
            # about 10 s of CPU work: a 128-row probe panel, then a panel of
            # whole 128-row blocks scaled to it
            _, dt0 = cpu_baseline(A, B, n, 128, threads)
            rows_s = int(min(n, max(128.0, 128.0 * 10.0 / max(dt0, 1e-3))) // 128 * 128)
        v, dt = cpu_baseline(A, B, n, rows_s, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{rows_s} x {n} x {n} row panel ({dt:.1f} s), oracle restatement of "
                         "pidblas::mulmm over the vblas sequential-chain dgemm (NEON "
                         "micro-kernel on aarch64)",
               "fp64_gflops": 4e3 * v}
        pk = host_fp64_peak_gflops(threads)
        cpu["host_fp64_peak"] = pk
        cpu["frac_of_host_fp64_peak"] = (4e3 * v / pk["gflops"]) if pk else None

    also = None
    if rank == 0 and not args.no_also:
        del dA, dB, dC
        torch.cuda.empty_cache()
        also = bench_also(dev, stream)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if form_name == "plain" else "bf16-slices/f64",
            "data": "synthetic (seeded)",
            "form": form_name, "slices": slices or "default", "slices_source": slices_src,
            "config": headline_config(n, ws),
            "plain": {"value": plain_tflops, "ms_per_step": plain_ms, "steps": args.plain_steps},
            "speedup_vs_plain": value / plain_tflops,
            "width_vs_plain": width,
            "containment_failures": fails, "containment_sample": 1024,
            "model_bitexact_sample": model,
            "auto_pick": auto_pick,
            "e2e": {"value": e2e_val, "unit": UNIT,
                    "h2d_bytes_per_step": e2e_h2d, "d2h_bytes_per_step": e2e_d2h,
                    "steps": e2e_steps, "step_ms": e2e_step_ms, "clocks": clk_e2e.summary()},
            "gpu_launches": int(launches),
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "also": also,
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


# DRAM bytes (read + write) of the oz_slice_gemm_kernel launch of one
# n = 8192 product at 8 slices with the fast radius products (2 x 3 radius
# digit pairs and 16 residue GEMMs in one launch), from a one-pass ncu
# capture of dram__bytes_read.sum and dram__bytes_write.sum on a GB300
# (21.30 + 2.06 GB).
GEMM_TRAFFIC_N8192 = 23.36e9


def ozaki_roofline(phases, tc_flops, steps, pk, pk_kind, n=8192, fast8=True):
    """Dominant kernel oz_slice_gemm_kernel (one launch per call for the
    default CRT form, three for the slice form): the algorithmic bf16 tensor
    flops (2 m n k per slice pair or modulus) over the summed CUDA-event time
    of its phases on the launching stream."""
    gemm_ms = sum(phases[1:4])
    phase_ms = {"prep": phases[0] / steps, "slice_gemm": gemm_ms / steps,
                "reassembly": phases[4] / steps}
    if phases[1] > 0 or phases[2] > 0:  # slice form: radius products run as launches of their own
        phase_ms.update(radius1=phases[1] / steps, radius2=phases[2] / steps,
                        midpoint=phases[3] / steps)
    achieved = tc_flops / (gemm_ms * 1e-3) / 1e12 if gemm_ms > 0 else None
    peak = pk.get("bf16_tflops", 1900.0)
    return {"bound": "tensor", "kernel": "oz_slice_gemm_kernel", "achieved": achieved,
            "peak": peak, "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
            "traffic": GEMM_TRAFFIC_N8192 if (n == 8192 and fast8) else None,
            "traffic_unit": "bytes per call (1 launch)",
            "peak_kind": f"{pk_kind} bf16 dense (burst); sustained {pk.get('bf16_tflops_sustained')}",
            "algorithmic": "2*m*n*k per bf16 product: L residue GEMMs + the radius digit "
                           "pairs (2 x 3 with the fast radius products, else 2 x 4)",
            "phase_ms_per_call": phase_ms}


# ---------------------------------------------------------------- other workloads
BATCH_WORKLOAD = ("batched interval GEMMs: {} problems, m,n,k log-uniform [32,1024], "
                  "mid U[-1,1], rad 1e-12|mid|")


def dev_intervals(count, gen, dev, rad_ratio=1e-12):
    """kv buffer of `count` intervals, mid U[-1, 1], rad rad_ratio |mid|."""
    import torch
    out = torch.empty(2 * count, dtype=torch.float64, device=dev)
    v = out.view(-1, 2)
    step = 1 << 26
    for a in range(0, count, step):
        b = min(count, a + step)
        mid = torch.rand(b - a, generator=gen, dtype=torch.float64, device=dev) * 2.0 - 1.0
        rad = mid.abs() * rad_ratio
        v[a:b, 0] = mid - rad
        v[a:b, 1] = mid + rad
    return out


def dev_ephi(count, phi, gen, dev):
    """E(phi) entries on the device: mantissa U[1, 2), random sign, exponent U{-phi..phi}."""
    import torch
    mant = 1.0 + torch.rand(count, generator=gen, dtype=torch.float64, device=dev)
    sign = torch.randint(0, 2, (count,), generator=gen, device=dev) * 2 - 1
    ex = torch.randint(-phi, phi + 1, (count,), generator=gen, device=dev)
    return torch.ldexp(mant * sign, ex.to(torch.float64))


def dev_dd(count, phi, gen, dev):
    """dd buffer: hi from E(phi), lo = hi 2^-53 u, u U[-1, 1]."""
    import torch
    hi = dev_ephi(count, phi, gen, dev)
    u = torch.rand(count, generator=gen, dtype=torch.float64, device=dev) * 2.0 - 1.0
    out = torch.empty(2 * count, dtype=torch.float64, device=dev)
    out.view(-1, 2)[:, 0] = hi
    out.view(-1, 2)[:, 1] = hi * 2.0 ** -53 * u
    return out


def time_stream(fn, stream, steps, warmup=1):
    import torch
    torch.cuda.synchronize()  # inputs are made on torch's stream, the work runs on `stream`
    for _ in range(warmup):
        fn()
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    stream.synchronize()
    return e0.elapsed_time(e1) / steps


def time_profiled(fn, stream, steps, pk):
    """time_stream plus the library's phase timing: (ms per call, roofline of
    the slice GEMMs against the measured bf16 burst peak)."""
    import torch
    from vcp_gb300 import _lib
    torch.cuda.synchronize()  # inputs are made on torch's stream, the work runs on `stream`
    fn()
    stream.synchronize()
    _lib.profile(True)
    _lib.profile_read()
    ms = time_stream(fn, stream, steps, warmup=0)
    phases, flops = _lib.profile_read()
    _lib.profile(False)
    gemm_ms = sum(phases[1:4])
    peak = pk.get("bf16_tflops", 1900.0)
    ach = flops / (gemm_ms * 1e-3) / 1e12 if gemm_ms > 0 else None
    return ms, {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                "frac": ach / peak if ach else None,
                "phase_ms_per_call": [p / steps for p in phases]}


def cpu_rate(fn, flops):
    t0 = time.perf_counter()
    fn()
    return flops / (time.perf_counter() - t0) / 1e12


def bench_batch(dev, stream, steps=1, count=4096, seed=4096, forms=("plain", "ozaki", "auto"),
                check=True):
    """Batched uneven interval GEMMs through captured CUDA graphs."""
    import torch
    from vcp_gb300 import batch, pidcuda
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    dims = np.exp(rng.uniform(np.log(32), np.log(1024), (count, 3))).round().astype(np.int64)
    m, n, k = dims[:, 0], dims[:, 1], dims[:, 2]
    na, nb, nc = m * k, k * n, m * n
    oa = np.concatenate([[0], np.cumsum(na)])
    ob = np.concatenate([[0], np.cumsum(nb)])
    oc = np.concatenate([[0], np.cumsum(nc)])
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    pa = dev_intervals(int(oa[-1]), gen, dev)
    pb = dev_intervals(int(ob[-1]), gen, dev)
    pc = torch.empty(2 * int(oc[-1]), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()  # the pools are written on torch's stream
    probs = [(int(m[i]), int(n[i]), int(k[i]), pa[2 * oa[i]:2 * oa[i + 1]], int(m[i]),
              pb[2 * ob[i]:2 * ob[i + 1]], int(k[i]), pc[2 * oc[i]:2 * oc[i + 1]], int(m[i]))
             for i in range(count)]
    flops = float(np.sum(2.0 * m * n * k))
    out = {"workload": BATCH_WORKLOAD.format(count), "problems": count, "gflop_per_batch": flops / 1e9,
           "seed": seed}
    codes = {"plain": pidcuda.FORM_PLAIN, "ozaki": pidcuda.FORM_OZAKI, "auto": pidcuda.FORM_AUTO}
    sample = rng.choice(count, 6, replace=False)
    widths = {}
    for name in forms:
        t0 = time.perf_counter()
        g = batch.BatchGraph(probs, codes[name], 0, stream)
        t_create = time.perf_counter() - t0
        ms = time_stream(lambda: g.launch(stream), stream, steps)
        _, lat = g.latencies(stream)
        rec = {"tflops": flops / (ms * 1e-3) / 1e12, "ms_per_batch": ms,
               "p50_us": float(np.percentile(lat, 50)), "p99_us": float(np.percentile(lat, 99)),
               "graph_create_s": t_create}
        if name == "auto":
            rec["problems_on_tensor_cores"] = int(sum(
                pidcuda.autotune_choice(int(m[i]), int(n[i]), int(k[i]), batched=True)
                != pidcuda.FORM_PLAIN
                for i in range(count)))
        if check:
            fails, ws = 0, []
            for i in sample:
                Ah = probs[i][3].cpu().numpy()
                Bh = probs[i][5].cpu().numpy()
                Ch = probs[i][7].cpu().numpy()
                mi, ni, ki = int(m[i]), int(n[i]), int(k[i])
                r = np.random.default_rng(i).integers(0, mi, 64)
                c = np.random.default_rng(i + 1).integers(0, ni, 64)
                lo, up = O.exact_hull(mi, ni, ki, Ah, Bh, r, c)
                idx = 2 * (r + c * mi)
                fails += int(np.sum(Ch[idx] > lo) + np.sum(Ch[idx + 1] < up))
                ws.append(Ch[1::2] - Ch[0::2])
            rec["containment_failures"] = fails
            rec["containment_sample"] = int(64 * len(sample))
            widths[name] = np.concatenate(ws)
        g.close()
        out[name] = rec
    if "plain" in widths and "ozaki" in widths:
        out["width_ozaki_vs_plain_median"] = float(np.median(widths["ozaki"] / widths["plain"]))
    # CPU: the oracle restatement of pidblas::mulmm on the first 64 problems
    sel = list(range(min(64, count)))
    hs = [(int(m[i]), int(n[i]), int(k[i]), probs[i][3].cpu().numpy(), probs[i][5].cpu().numpy())
          for i in sel]
    fl_s = float(sum(2.0 * a * b * c for (a, b, c, _, _) in hs))
    out["cpu_baseline"] = {
        "value": cpu_rate(lambda: [O.pidblas_mulmm(a, b, c, Ah_, Bh_, cpu_count())
                                   for (a, b, c, Ah_, Bh_) in hs], fl_s),
        "unit": "TFLOP/s", "cores": cpu_count(), "kind": "port",
        "sample": f"the first {len(sel)} problems, oracle restatement of pidblas::mulmm"}
    del pa, pb, pc
    return out


def bench_dd(dev, stream, n, phi, steps=2, seed=77, sample=256, cpu_rows=0):
    import torch
    from vcp_gb300 import pddcuda
    from oracle import oracle as O
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed + n + phi)
    A = dev_dd(n * n, phi, gen, dev)
    B = dev_dd(n * n, phi, gen, dev)
    C = torch.empty(2 * n * n, dtype=torch.float64, device=dev)
    E = torch.empty(n * n, dtype=torch.float64, device=dev)
    ms, roof = time_profiled(lambda: pddcuda.mulmm_dev(n, n, n, A, n, B, n, C, n, E, n, 0, stream),
                             stream, steps, peaks()[0])
    Ah, Bh, Ch, Eh = (t.cpu().numpy() for t in (A, B, C, E))
    rs = np.random.default_rng(seed)
    r = rs.integers(0, n, sample)
    c = rs.integers(0, n, sample)
    err, ab = O.dd_residual(n, n, n, Ah, Bh, Ch, r, c)
    bnd = Eh[r + c * n]
    rel = err / np.where(ab > 0, ab, 1.0)
    nz = err > 0
    out = {"n": n, "phi": phi, "tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12, "ms": ms,
           "rel_err_max": float(rel.max()), "rel_err_median": float(np.median(rel)),
           "bound_failures": int(np.sum(err > bnd)),
           "bound_over_err_median": float(np.median(bnd[nz] / err[nz])) if nz.any() else None,
           "bound_rel_median": float(np.median(bnd / np.where(ab > 0, ab, 1.0))),
           "sample": sample, "slices": "default (14, w = 112)", "roofline": roof}
    if cpu_rows:
        # pddblas::mulmm (oracle restatement: Ozaki slices, RN dgemm, dd sums)
        # on a row panel: its time and, on the panel's entries, its error
        # next to the GPU's
        Ap = np.ascontiguousarray(Ah.reshape(n, n, 2)[:, :cpu_rows, :]).ravel()
        t0 = time.perf_counter()
        Pp = O.pddblas_mulmm(cpu_rows, n, n, Ap, Bh, cpu_count())
        dt = time.perf_counter() - t0
        pr = rs.integers(0, cpu_rows, sample).astype(np.int32)
        pc = rs.integers(0, n, sample).astype(np.int32)
        ep, abp = O.dd_residual(cpu_rows, n, n, Ap, Bh, Pp, pr, pc)
        Cp = np.ascontiguousarray(Ch.reshape(n, n, 2)[:, :cpu_rows, :]).ravel()
        eg, _ = O.dd_residual(cpu_rows, n, n, Ap, Bh, Cp, pr, pc)
        sc = np.where(abp > 0, abp, 1.0)
        out["cpu_baseline"] = {"value": 2.0 * cpu_rows * n * n / dt / 1e12, "unit": "TFLOP/s",
                               "cores": cpu_count(), "kind": "port",
                               "sample": f"{cpu_rows} x {n} x {n} row panel ({dt:.2f} s), "
                                         "oracle restatement of pddblas::mulmm"}
        out["accuracy_vs_pddblas"] = {
            "entries": sample, "gpu_rel_err_median": float(np.median(eg / sc)),
            "gpu_rel_err_max": float(np.max(eg / sc)),
            "pddblas_rel_err_median": float(np.median(ep / sc)),
            "pddblas_rel_err_max": float(np.max(ep / sc))}
    return out


def bench_point(dev, stream, m, n, k, phi, slice_list, steps=2, plain=True, seed=11,
                sample=256):
    """udmatmul shape (vblas naming: A m x n, B n x k)."""
    import torch
    from vcp_gb300 import vblas
    from oracle import oracle as O
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed + m + n + k + phi)
    A = dev_ephi(m * n, phi, gen, dev)
    B = dev_ephi(n * k, phi, gen, dev)
    CU = torch.empty(m * k, dtype=torch.float64, device=dev)
    CD = torch.empty_like(CU)
    fl = 2.0 * m * n * k
    rs = np.random.default_rng(seed)
    r = rs.integers(0, m, sample)
    c = rs.integers(0, k, sample)
    Ah, Bh = A.cpu().numpy(), B.cpu().numpy()
    dn, up = O.exact_dot(m, k, n, Ah, Bh, r, c)
    idx = r + c * m
    out = {"m": m, "n": n, "k": k, "phi": phi}
    wp = None
    if plain:
        ms = time_stream(lambda: vblas.udmatmul_dev(m, n, k, A, m, B, n, CU, CD, m, stream),
                         stream, steps)
        u, d = CU.cpu().numpy(), CD.cpu().numpy()
        wp = u - d
        out["plain"] = {"tflops": fl / (ms * 1e-3) / 1e12, "ms": ms,
                        "containment_failures": int(np.sum(d[idx] > dn) + np.sum(u[idx] < up)),
                        "fp64_tflops": 2 * fl / (ms * 1e-3) / 1e12}
        # CPU: the oracle restatement of vblas rmatmul (one direction) on a row panel
        rows = max(1, min(m, int(2e10 / (2.0 * n * k))))
        Ap = Ah.reshape(n, m)[:, :rows].copy().reshape(-1)
        out["cpu_baseline"] = {
            "value": cpu_rate(lambda: O.rmatmul(rows, n, k, Ap, Bh, 1, cpu_count()),
                              2.0 * rows * n * k),
            "unit": "TFLOP/s (one direction)", "cores": cpu_count(), "kind": "port",
            "sample": f"{rows} x {n} x {k} row panel, oracle restatement of vblas rmatmul"}
    for s_ in slice_list:
        ms, roof = time_profiled(lambda: vblas.udmatmul_ozaki_dev(m, n, k, A, m, B, n, CU, CD, m,
                                                                  s_, stream),
                                 stream, steps, peaks()[0])
        u, d = CU.cpu().numpy(), CD.cpu().numpy()
        rec = {"tflops": fl / (ms * 1e-3) / 1e12, "ms": ms, "roofline": roof,
               "containment_failures": int(np.sum(d[idx] > dn) + np.sum(u[idx] < up))}
        if wp is not None:
            ok = wp > 0
            rec["width_vs_plain_median"] = float(np.median((u - d)[ok] / wp[ok]))
        out[f"ozaki_s{s_}"] = rec
    return out


def _setup_inv(M):
    """Approximate inverse for a workload's setup (untimed): torch's linalg
    on the device, numpy on the host when that library cannot be loaded."""
    import torch
    try:
        return torch.linalg.inv(M)
    except RuntimeError:
        return torch.from_numpy(np.linalg.inv(M.cpu().numpy())).to(M.device)


def bench_lss(dev, stream, n, nrhs=1, steps=2, plain_steps=1, seed=91, cpu_n=768,
              forms=("plain", "ozaki"), cpu=True):
    """The verification of imats::linearsolve (vcpcu_ilss_verify) at n x n,
    nrhs right-hand sides: A = I + U[-1,1]/sqrt(n) (well conditioned), b
    U[-1,1], radii 2^-40 |mid|; R and mx formed on the device in FP64
    (setup, untimed).  Time per verification (four interval products, the
    norms, the enclosure), plain vs tensor-core form; the CPU leg is the
    oracle's restatement of the same steps at cpu_n (its time scaled by
    (n / cpu_n)^3, the R [A] product's share)."""
    import torch
    from vcp_gb300 import pidcuda
    from oracle import oracle as O
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed + n)

    def system(nn):
        mid = torch.rand(nn, nn, generator=gen, device=dev, dtype=torch.float64) * 2 - 1
        mid = mid / nn ** 0.5 + torch.eye(nn, device=dev, dtype=torch.float64)
        bm = torch.rand(nn, nrhs, generator=gen, device=dev, dtype=torch.float64) * 2 - 1

        def kv(m):
            r = m.abs() * 2.0 ** -40
            return torch.stack((m - r, m + r), dim=-1).transpose(0, 1).contiguous().reshape(-1)

        R = _setup_inv(mid)
        mx = R @ bm
        return (kv(mid), kv(bm), R.t().contiguous().reshape(-1),
                mx.t().contiguous().reshape(-1))

    A, b, R, mx = system(n)
    torch.cuda.synchronize()  # set up on the current stream, verified on `stream`
    x = torch.empty(2 * n * nrhs, dtype=torch.float64, device=dev)
    G = torch.empty(1, dtype=torch.float64, device=dev)
    out = {"n": n, "nrhs": nrhs}
    res = {}
    for name, form, st_ in (("plain", pidcuda.FORM_PLAIN, plain_steps),
                            ("ozaki", pidcuda.FORM_OZAKI, steps)):
        if name not in forms:
            continue
        ms = time_stream(lambda: pidcuda.linearsolve_verify_dev(
            n, nrhs, A, n, b, n, R, n, mx, n, x, n, G, form=form, stream=stream), stream, st_)
        res[name] = (x.cpu().numpy(), float(G.cpu()[0]))
        out[name] = {"ms": ms, "tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12,
                     "bound_RA_minus_I": res[name][1]}
    if len(res) == 2:
        xp, xo = res["plain"][0], res["ozaki"][0]
        wp, wo = xp[1::2] - xp[0::2], xo[1::2] - xo[0::2]
        out["width_ozaki_vs_plain_median"] = float(np.median(wo / wp))
        out["width_ozaki_vs_plain_max"] = float(np.max(wo / wp))
        out["speedup_ozaki_vs_plain"] = out["plain"]["ms"] / out["ozaki"]["ms"]
    if not cpu:
        return out
    # CPU: the restatement of the same steps at cpu_n, scaled by (n / cpu_n)^3
    Ac, bc, Rc, mc = (t.cpu().numpy() for t in system(cpu_n))
    t0 = time.perf_counter()
    st, _, _ = O.ilss_verify(cpu_n, nrhs, Ac, bc, Rc, mc, threads=cpu_count())
    dt = time.perf_counter() - t0
    out["cpu_baseline"] = {"ms_scaled": dt * 1e3 * (n / cpu_n) ** 3, "ms_sample": dt * 1e3,
                           "status": st, "cores": cpu_count(), "kind": "port",
                           "sample": f"n = {cpu_n}, nrhs = {nrhs}, oracle restatement of "
                                     f"imats::linearsolve's verification, time x (n/{cpu_n})^3"}
    return out


def bench_eig(dev, stream, n, steps=2, plain_steps=1, seed=93, forms=("plain", "ozaki")):
    """The verification of imats::eigsymge (vcpcu_ieigsymge stages 1 and 2)
    for A x = l B x, n x n: A symmetric N(0, 1/n), B = I + 0.1 G (G G^T form,
    positive definite), radii 2^-40 |mid|; the approximate eigenpairs and
    Y = inv(mid(B X)) formed on the device in FP64 beforehand (setup, as the
    reference takes them from LAPACK).  Time of the two stages (four n^3
    interval products, norms, enclosures), plain vs tensor-core form."""
    import torch
    from vcp_gb300 import pidcuda
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed + n)
    f64 = dict(dtype=torch.float64, device=dev)
    Am = torch.randn(n, n, generator=gen, **f64) / n ** 0.5
    Am = (Am + Am.t()) / 2
    G = torch.eye(n, **f64) + 0.1 * torch.randn(n, n, generator=gen, **f64) / n ** 0.5
    Bm = G @ G.t()
    Bm = (Bm + Bm.t()) / 2
    try:
        L = torch.linalg.cholesky(Bm)
        Li = torch.linalg.inv(L)
        w, V = torch.linalg.eigh(Li @ Am @ Li.t())
    except RuntimeError:  # torch's linalg library not loadable (e.g. under a profiler)
        Ln = np.linalg.cholesky(Bm.cpu().numpy())
        Lin = np.linalg.inv(Ln)
        wn, Vn = np.linalg.eigh(Lin @ Am.cpu().numpy() @ Lin.T)
        Li, w, V = (torch.from_numpy(v).to(dev) for v in (Lin, wn, Vn))
    X = (Li.t() @ V).t().contiguous().reshape(-1)

    def kv(m):
        r = m.abs() * 2.0 ** -40
        return torch.stack((m - r, m + r), dim=-1).transpose(0, 1).contiguous().reshape(-1)

    A, B = kv(Am), kv(Bm)
    C = torch.empty(2 * n * n, **f64)
    BX = torch.empty_like(C)
    M = torch.empty(n * n, **f64)
    # the setup ran on the current stream, the stages run on `stream`
    torch.cuda.synchronize()
    pidcuda.eigsymge_stage1_dev(n, A, n, B, n, X, n, C, BX, M, pidcuda.FORM_OZAKI, 0, stream)
    stream.synchronize()
    Y = _setup_inv(M.reshape(n, n).t()).t().contiguous().reshape(-1)
    torch.cuda.synchronize()
    lam = torch.empty(2 * n, **f64)
    bound = torch.empty(1, **f64)
    out = {"n": n}
    res = {}
    for name, form, st_ in (("plain", pidcuda.FORM_PLAIN, plain_steps),
                            ("ozaki", pidcuda.FORM_OZAKI, steps)):
        if name not in forms:
            continue

        def step():
            pidcuda.eigsymge_stage1_dev(n, A, n, B, n, X, n, C, BX, M, form, 0, stream)
            pidcuda.eigsymge_stage2_dev(n, w, Y, n, C, BX, lam, bound, form, 0, stream)
        ms = time_stream(step, stream, st_)
        res[name] = lam.cpu().numpy()
        out[name] = {"ms": ms, "bound_YBX_minus_I": float(bound.cpu()[0])}
    if len(res) == 2:
        wp = res["plain"][1::2] - res["plain"][0::2]
        wo = res["ozaki"][1::2] - res["ozaki"][0::2]
        out["width_ozaki_vs_plain_median"] = float(np.median(wo / wp))
        out["speedup_ozaki_vs_plain"] = out["plain"]["ms"] / out["ozaki"]["ms"]
        out["enclosure_width_median"] = float(np.median(wo))
    return out


def bench_cfg1(dev, stream, n=512, steps=3, seed=5):
    """cfg1: the n = 512 interval product, CPU (the oracle port of
    pidblas::mulmm, all host cores) against the GPU's plain form (every bit
    compared) and its tensor-core form; mid E(4), radius 2^-40 |mid|."""
    import torch
    from vcp_gb300 import pidcuda, workloads as W
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    A = W.interval_ephi(rng, n, n, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, n, n, 4, 2.0 ** -40)
    t0 = time.perf_counter()
    C_cpu = O.pidblas_mulmm(n, n, n, A, B, cpu_count())
    cpu_ms = (time.perf_counter() - t0) * 1e3
    dA, dB = (torch.from_numpy(v).to(dev) for v in (A, B))
    dC = torch.empty(2 * n * n, dtype=torch.float64, device=dev)
    out = {"n": n, "cpu_port_ms": cpu_ms, "cpu_cores": cpu_count()}
    for name, form in (("plain", pidcuda.FORM_PLAIN), ("ozaki", pidcuda.FORM_OZAKI)):
        ms = time_stream(lambda: pidcuda.mulmm_dev(n, n, n, dA, n, dB, n, dC, n, form, 0, stream),
                         stream, steps)
        out[name] = {"ms": ms, "tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12}
        if name == "plain":
            out[name]["bit_identical_to_cpu"] = bool(
                np.array_equal(dC.cpu().numpy().view(np.int64), C_cpu.view(np.int64)))
    out["speedup_plain_vs_cpu"] = cpu_ms / out["plain"]["ms"]
    return out


def bench_emden(dev, Ms=(30, 50, 70), cpu_Ms=(30,), repeats=2, forms=("plain", "ozaki")):
    """End-to-end Emden verification (-Laplace u = u^2 on the unit square,
    test_PDE/test_Emden.cpp): Newton on the GPU (FP64), then the
    verification in the plain and in the tensor-core form from the same
    Newton solution; the CPU pipeline (oracle products, all host cores) on
    the orders in cpu_Ms.  Wall times are of the last of `repeats` runs."""
    import torch
    from vcp_gb300 import emden as E
    from vcp_gb300 import legendre, pidcuda
    cases = []
    for M in Ms:
        rec = {"M": M, "n": ((M + 1) // 2) ** 2,
               "points_per_dim": [E.npts_inverse(M), E.npts_residual(M)]}
        t0 = time.perf_counter()
        legendre.basis_tables(M, E.npts_inverse(M))
        legendre.basis_tables(M, E.npts_residual(M))
        E.stiffness(M, *E.even_list(M))
        rec["legendre_tables_s"] = time.perf_counter() - t0
        g = E.GpuProducts(pidcuda.FORM_PLAIN)
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            c, it, step = E.newton(M, g)
            torch.cuda.synchronize()
            rec["newton"] = {"s": time.perf_counter() - t0, "iterations": it, "last_step": step}
        for name, form in (("plain", pidcuda.FORM_PLAIN), ("ozaki", pidcuda.FORM_OZAKI)):
            if name not in forms:
                continue
            for _ in range(repeats):
                r = E.verify(M, E.GpuProducts(form), c=c, newton_info=(it, step))
            d = r.as_dict()
            t_up = d["seconds"]["uhphiphi_product"]
            rec[name] = {k: d[k] for k in ("verified", "error_bound_H10", "K", "residual_L2",
                                           "residual_Hm1", "kantorovich", "uh_max",
                                           "lambda_min", "lambda_max", "CN", "Cs3")}
            rec[name]["seconds"] = d["seconds"]
            rec[name]["verification_s"] = d["seconds"]["total"] - d["seconds"]["newton"]
            rec[name]["uhphiphi_tflops"] = d["sizes"]["uhphiphi_flops"] / t_up / 1e12
            torch.cuda.empty_cache()
        if "plain" in rec and "ozaki" in rec:
            rec["bound_ozaki_over_plain"] = rec["ozaki"]["error_bound_H10"] / \
                rec["plain"]["error_bound_H10"]
            rec["verification_speedup_ozaki_vs_plain"] = rec["plain"]["verification_s"] / \
                rec["ozaki"]["verification_s"]
        if M in cpu_Ms:
            from oracle.emden_host import HostProducts
            hp = HostProducts(cpu_count())
            t0 = time.perf_counter()
            cc, itc, stc = E.newton(M, hp)
            rc = E.verify(M, hp, c=cc, newton_info=(itc, stc))
            d = rc.as_dict()
            rec["cpu"] = {k: d[k] for k in ("verified", "error_bound_H10", "K", "residual_L2")}
            rec["cpu"].update({"wall_s": time.perf_counter() - t0, "cores": cpu_count(),
                               "kind": "port", "seconds": d["seconds"]})
        cases.append(rec)
    return {"cases": cases}


def parse_list(text, default, conv=int):
    return [conv(x) for x in text.split(",") if x] if text else default


def run_workload(args, dev, stream):
    """--workload batch | dd | point: one JSON line at that workload's sizes."""
    import torch
    from vcp_gb300 import pidcuda
    t0 = time.perf_counter()
    with ClockSampler(dev.index or 0) as clk:
        if args.workload == "batch":
            pidcuda.autotune(stream)
            forms = ("ozaki",) if args.form == "ozaki" else ("plain", "ozaki", "auto")
            res = bench_batch(dev, stream, steps=args.steps, count=args.batch_count, forms=forms,
                              check=not args.no_cpu)
            metric, unit = "batched interval GEMM TFLOP/s (4096 uneven problems)", "TFLOP/s"
            value = res["ozaki"]["tflops"]
        elif args.workload == "lss":
            forms = ("ozaki",) if args.form == "ozaki" else ("plain", "ozaki")
            res = {"cases": [bench_lss(dev, stream, n, nrhs, steps=args.steps, forms=forms,
                                       cpu=not args.no_cpu)
                             for n in parse_list(args.sizes, [8192])
                             for nrhs in parse_list(args.phis, [1])]}
            metric, unit = ("verified linear solve, device-resident verification "
                            "(imats::linearsolve after R, mx): ms"), "ms"
            value = min(c["ozaki"]["ms"] for c in res["cases"])
        elif args.workload == "eig":
            forms = ("ozaki",) if args.form == "ozaki" else ("plain", "ozaki")
            res = {"cases": [bench_eig(dev, stream, n, steps=args.steps, forms=forms)
                             for n in parse_list(args.sizes, [4096])]}
            metric, unit = ("verified generalized symmetric eigenvalues, device-resident "
                            "verification (imats::eigsymge after X, lambda, Y): ms"), "ms"
            value = min(c["ozaki"]["ms"] for c in res["cases"])
        elif args.workload == "emden":
            res = bench_emden(dev, tuple(parse_list(args.sizes, [30, 50, 70])),
                              () if args.no_cpu else (30, 50),
                              forms=("ozaki",) if args.form == "ozaki" else ("plain", "ozaki"))
            metric, unit = ("Emden verification wall time (s), tensor-core form, "
                            "largest order"), "s"
            value = res["cases"][-1]["ozaki"]["verification_s"]
        elif args.workload == "dd":
            res = {"cases": [bench_dd(dev, stream, n, phi, steps=args.steps,
                                      cpu_rows=0 if args.no_cpu else (64 if n <= 2048 else 16))
                             for n in parse_list(args.sizes, [2048, 8192])
                             for phi in parse_list(args.phis, [0, 16])]}
            metric, unit = "dd GEMM TFLOP/s (pddblas semantics)", "TFLOP/s"
            value = max(c["tflops"] for c in res["cases"])
        else:
            shapes = []
            for tok in (args.sizes.split(",") if args.sizes else
                        ["1024", "4096", "8192", "16384", "16384:16384:256"]):
                dims = [int(x) for x in tok.split(":")]
                shapes.append(tuple(dims) if len(dims) == 3 else (dims[0],) * 3)
            cases = []
            for (m_, n_, k_) in shapes:
                for phi in parse_list(args.phis, [0, 8, 32]):
                    cases.append(bench_point(dev, stream, m_, n_, k_, phi,
                                             parse_list(args.slice_list, [4, 5, 6, 7, 8, 9]),
                                             steps=args.steps))
                    torch.cuda.empty_cache()
            res = {"cases": cases}
            metric, unit = "up/down point GEMM TFLOP/s: Ozaki enclosure vs FP64 RU/RD", "TFLOP/s"
            value = None
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "workload": args.workload, "data": "synthetic (seeded)", "results": res,
            "wall_s": time.perf_counter() - t0, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def bench_also(dev, stream):
    """Short runs of the other workloads for the headline line."""
    from vcp_gb300 import pidcuda
    out = {}
    for key, fn in (("autotune", lambda: pidcuda.autotune(stream)),
                    ("batch", lambda: bench_batch(dev, stream, steps=1)),
                    ("dd", lambda: [bench_dd(dev, stream, 8192, 0, steps=2, cpu_rows=16),
                                    bench_dd(dev, stream, 8192, 16, steps=2, cpu_rows=0)]),
                    ("cfg1", lambda: bench_cfg1(dev, stream)),
                    ("lss", lambda: bench_lss(dev, stream, 8192, 1, steps=3)),
                    ("eig", lambda: bench_eig(dev, stream, 2048, steps=3)),
                    ("point", lambda: bench_point(dev, stream, 8192, 8192, 8192, 0, [6, 8],
                                                  steps=2)),
                    ("emden", lambda: bench_emden(dev, (30, 50), (30,)))):
        t0 = time.perf_counter()
        try:
            out[key] = fn()
        except Exception as e:  # reported, the headline line still prints
            out[key] = {"error": f"{type(e).__name__}: {e}"}
        if isinstance(out[key], dict):
            out[key]["wall_s"] = time.perf_counter() - t0
        elif isinstance(out[key], list):
            out[key] = {"cases": out[key], "wall_s": time.perf_counter() - t0}
    return out


def main():
    args = parse()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.workload != "interval":
        import torch
        from vcp_gb300.build import build
        if rank == 0:
            build()
        barrier(ws)
        torch.cuda.set_device(local)
        dev = torch.device("cuda", local)
        if rank == 0:
            run_workload(args, dev, torch.cuda.Stream(device=dev))
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
