"""GPU tests of the batched interval GEMMs (one persistent grouped launch for
the plain form; CUDA-graph capture and replay): every problem is
bit-identical to the same product through vcpcu_igemm_dev in the same form,
graph replays reproduce the result, and per-problem latencies are reported."""
import numpy as np
import pytest

from vcp_gb300 import batch, pidcuda
from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def make_batch(rng, count, lo=1, hi=200):
    import torch
    probs, refs = [], []
    for _ in range(count):
        m, n, k = (int(x) for x in np.exp(rng.uniform(np.log(lo), np.log(hi), 3)).round())
        A = torch.from_numpy(W.interval_uniform(rng, m, k, 1e-12)).cuda()
        B = torch.from_numpy(W.interval_uniform(rng, k, n, 1e-12)).cuda()
        C = torch.full((2 * m * n,), float("nan"), dtype=torch.float64, device="cuda")
        probs.append((m, n, k, A, m, B, k, C, m))
    return probs


@pytest.mark.parametrize("form", [pidcuda.FORM_PLAIN, pidcuda.FORM_OZAKI])
def test_batched_matches_single_products(cuda_lib, form):
    import torch
    rng = np.random.default_rng(form + 1)
    probs = make_batch(rng, 40)
    batch.run(probs, form)
    torch.cuda.synchronize()
    for (m, n, k, A, lda, B, ldb, C, ldc) in probs:
        ref = torch.empty_like(C)
        pidcuda.mulmm_dev(m, n, k, A, lda, B, ldb, ref, ldc, form)
        torch.cuda.synchronize()
        assert torch.equal(C.view(torch.int64), ref.view(torch.int64)), (m, n, k)


@pytest.mark.parametrize("form", [pidcuda.FORM_PLAIN, pidcuda.FORM_OZAKI])
def test_batch_graph_replay_and_latencies(cuda_lib, form):
    import torch
    rng = np.random.default_rng(10 + form)
    probs = make_batch(rng, 25, 16, 300)
    g = batch.BatchGraph(probs, form)
    g.launch()
    torch.cuda.synchronize()
    first = [p[7].clone() for p in probs]
    for p in probs:
        p[7].fill_(0.0)
    g.launch()
    start, lat = g.latencies()
    for p, f in zip(probs, first):
        assert torch.equal(p[7].view(torch.int64), f.view(torch.int64))
    assert np.all(lat > 0) and np.all(start >= 0)
    g.close()


def test_grouped_tensor_core_batch_edges(cuda_lib):
    """The grouped tensor-core path (buckets of equal padded K, stacked
    operand planes) on problems spanning several tiles and chunks, with empty
    and k = 0 problems mixed in: every product bit-identical to its single
    call."""
    import torch
    rng = np.random.default_rng(77)
    shapes = [(1100, 300, 2100), (130, 600, 1030), (5, 7, 0), (0, 9, 12), (64, 1, 64),
              (257, 513, 64), (40, 40, 40), (129, 257, 1025), (3, 900, 7)]
    probs = []
    for (m, n, k) in shapes:
        A = torch.from_numpy(W.interval_uniform(rng, max(m, 1), max(k, 1), 1e-12)).cuda()
        B = torch.from_numpy(W.interval_uniform(rng, max(k, 1), max(n, 1), 1e-12)).cuda()
        C = torch.full((2 * max(m, 1) * max(n, 1),), float("nan"), dtype=torch.float64,
                       device="cuda")
        probs.append((m, n, k, A, max(m, 1), B, max(k, 1), C, max(m, 1)))
    batch.run(probs, pidcuda.FORM_OZAKI)
    torch.cuda.synchronize()
    for (m, n, k, A, lda, B, ldb, C, ldc) in probs:
        if m == 0 or n == 0:
            continue
        ref = torch.empty_like(C)
        pidcuda.mulmm_dev(m, n, k, A, lda, B, ldb, ref, ldc, pidcuda.FORM_OZAKI)
        torch.cuda.synchronize()
        assert torch.equal(C.view(torch.int64), ref.view(torch.int64)), (m, n, k)


@pytest.mark.parametrize("slices", [2, 10])
def test_grouped_batch_slice_counts(cuda_lib, slices):
    """The grouped tensor-core path at other precisions: 2 slices (14-bit
    operands, few moduli) and 10 slices (62-bit operands: the 12-bit limb
    forms of the splits); every product bit-identical to its single call."""
    import torch
    rng = np.random.default_rng(90 + slices)
    probs = make_batch(rng, 30, 20, 400)
    batch.run(probs, pidcuda.FORM_OZAKI, slices)
    torch.cuda.synchronize()
    for (m, n, k, A, lda, B, ldb, C, ldc) in probs:
        ref = torch.empty_like(C)
        pidcuda.mulmm_dev(m, n, k, A, lda, B, ldb, ref, ldc, pidcuda.FORM_OZAKI, slices)
        torch.cuda.synchronize()
        assert torch.equal(C.view(torch.int64), ref.view(torch.int64)), (m, n, k, slices)


def test_grouped_batch_chunked_buckets(cuda_lib):
    """A bucket (one padded K) holding more work than one chunk is cut into
    several chunks that run one after another on the shared workspace: 200
    problems of k <= 64 (padded K 64; 14 or 15 moduli by k) and m, n in
    [200, 400] make two buckets of about 0.45 ms of estimated work each, two
    chunks apiece; every product bit-identical to its single call, and graph
    replays give each problem a latency."""
    import torch
    rng = np.random.default_rng(123)
    probs = []
    for _ in range(200):
        m, n = (int(x) for x in rng.integers(200, 401, 2))
        k = int(rng.integers(1, 65))
        A = torch.from_numpy(W.interval_uniform(rng, m, k, 1e-12)).cuda()
        B = torch.from_numpy(W.interval_uniform(rng, k, n, 1e-12)).cuda()
        C = torch.full((2 * m * n,), float("nan"), dtype=torch.float64, device="cuda")
        probs.append((m, n, k, A, m, B, k, C, m))
    g = batch.BatchGraph(probs, pidcuda.FORM_OZAKI)
    g.launch()
    _, lat = g.latencies()
    assert np.all(lat > 0)
    g.close()
    for (m, n, k, A, lda, B, ldb, C, ldc) in probs:
        ref = torch.empty_like(C)
        pidcuda.mulmm_dev(m, n, k, A, lda, B, ldb, ref, ldc, pidcuda.FORM_OZAKI)
        torch.cuda.synchronize()
        assert torch.equal(C.view(torch.int64), ref.view(torch.int64)), (m, n, k)
