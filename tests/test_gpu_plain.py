"""GPU parity of the plain FP64 form through the C ABI.

* vcpcu_rmatmul / vcpcu_udmatmul are bit-identical to the oracle's vblas
  rmatmul restatement (which is itself pinned bit-for-bit to the reference
  and its golden vectors), over ragged shapes, all three rounding modes and
  the vblas edge cases (m or k = 0: no-op; inner n = 0: zeros);
* the vblas known-answer rounding tests (vblas/Check_rmatmul_rounding.cpp,
  vblas/Check_udmatmul_rounding.cpp);
* vcpcu_igemm (plain form) is bit-identical to the pidblas::mulmm
  restatement and encloses the exact interval hull (long accumulator).
"""
from pathlib import Path

import numpy as np
import pytest

from vcp_gb300 import pidcuda, vblas
from vcp_gb300 import workloads as W
from vcp_gb300.errors import DimensionError

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


SHAPES = [(1, 1, 1), (1, 7, 1), (7, 1, 9), (33, 17, 65), (64, 64, 64), (65, 129, 63),
          (129, 16, 200), (5, 1000, 3), (200, 3, 130)]


@pytest.mark.parametrize("shape", SHAPES)
def test_rmatmul_bitexact(cuda_lib, oracle, shape):
    m, n, k = shape
    rng = np.random.default_rng(m * 1000 + n * 10 + k)
    for phi in (0, 8, 32):
        A, B = W.ephi(rng, m * n, phi), W.ephi(rng, n * k, phi)
        for rnd in (1, -1, 0, 7):
            C = np.full(m * k, np.nan)
            vblas.rmatmul(m, n, k, A, B, C, rnd)
            ref = oracle.rmatmul(m, n, k, A, B, rnd)
            assert np.array_equal(bits(C), bits(ref)), (shape, phi, rnd)


def test_rmatmul_golden(cuda_lib):
    g = np.load(GOLDEN)
    for idx in range(int(g["n_rm"][0])):
        m, n, k = map(int, g[f"rm{idx}_shape"])
        for rnd, tag in ((1, "up"), (-1, "dn"), (0, "rn")):
            C = np.empty(m * k)
            vblas.rmatmul(m, n, k, g[f"rm{idx}_A"], g[f"rm{idx}_B"], C, rnd)
            assert np.array_equal(bits(C), bits(g[f"rm{idx}_{tag}"])), (idx, tag)


def test_udmatmul_bitexact(cuda_lib, oracle):
    rng = np.random.default_rng(11)
    for m, n, k in [(70, 90, 33), (1, 300, 1), (128, 128, 128)]:
        A, B = W.ephi(rng, m * n, 8), W.ephi(rng, n * k, 8)
        CU, CD = np.empty(m * k), np.empty(m * k)
        vblas.udmatmul(m, n, k, A, B, CU, CD)
        assert np.array_equal(bits(CU), bits(oracle.rmatmul(m, n, k, A, B, 1)))
        assert np.array_equal(bits(CD), bits(oracle.rmatmul(m, n, k, A, B, -1)))


def test_rmatmul_edge_cases(cuda_lib):
    C = np.full(6, 7.0)
    vblas.rmatmul(0, 3, 2, np.zeros(3), np.zeros(6), C, 1)  # m = 0: untouched
    vblas.rmatmul(3, 3, 0, np.zeros(9), np.zeros(3), C, 1)  # k = 0: untouched
    assert np.all(C == 7.0)
    vblas.rmatmul(3, 0, 2, np.zeros(1), np.zeros(1), C, 1)  # inner n = 0: zeroed
    assert np.all(C == 0.0) and not np.any(np.signbit(C))
    with pytest.raises(DimensionError):
        from vcp_gb300 import _lib
        _lib.call("vcpcu_rmatmul_dev", 4, 4, 4, 1, 2, 1, 4, 1, 4, 1, None)  # lda < m


def test_rounding_kat(cuda_lib):
    """vblas/Check_rmatmul_rounding.cpp at its own size n = 450, every i."""
    n = 450
    A = np.zeros((n, n)); B = np.zeros((n, n))
    for i in range(0, n, 7):
        A[:] = 0; B[:] = 0
        A[:, i] = 1.0 / 3.0; B[i, :] = 1.0 / 3.0
        a, b = A.ravel(order="F"), B.ravel(order="F")
        CU, CD = np.empty(n * n), np.empty(n * n)
        vblas.rmatmul(n, n, n, a, b, CU, 1)
        vblas.rmatmul(n, n, n, a, b, CD, -1)
        assert np.all(CU != CD), i
    for i in range(2, n, 11):
        A[:] = 0; B[:] = 0
        A[:, 1] = 1.0; B[1, :] = 1.0
        A[:, i] = 2.0 ** -27; B[i, :] = 2.0 ** -27
        a, b = A.ravel(order="F"), B.ravel(order="F")
        CU, CD = np.empty(n * n), np.empty(n * n)
        vblas.udmatmul(n, n, n, a, b, CU, CD)
        assert np.all(CU > CD), i


def test_rmatmul_dev_leading_dims(cuda_lib, oracle):
    import torch
    rng = np.random.default_rng(12)
    m, n, k, lda, ldb, ldc = 50, 70, 30, 64, 80, 57
    Af = np.zeros(lda * n); Bf = np.zeros(ldb * k)
    A, B = W.ephi(rng, m * n, 4), W.ephi(rng, n * k, 4)
    for p in range(n):
        Af[p * lda:p * lda + m] = A[p * m:(p + 1) * m]
    for j in range(k):
        Bf[j * ldb:j * ldb + n] = B[j * n:(j + 1) * n]
    dA = torch.from_numpy(Af).cuda(); dB = torch.from_numpy(Bf).cuda()
    dC = torch.full((ldc * k,), float("nan"), dtype=torch.float64, device="cuda")
    vblas.rmatmul_dev(m, n, k, dA, lda, dB, ldb, dC, ldc, -1)
    torch.cuda.synchronize()
    C = dC.cpu().numpy().reshape(k, ldc)[:, :m].ravel()
    assert np.array_equal(bits(C), bits(oracle.rmatmul(m, n, k, A, B, -1)))
    assert np.all(np.isnan(dC.cpu().numpy().reshape(k, ldc)[:, m:]))


ISHAPES = [(1, 1, 1), (5, 4, 6), (64, 64, 64), (65, 33, 129), (128, 96, 17), (3, 200, 70)]


@pytest.mark.parametrize("shape", ISHAPES)
def test_igemm_plain_bitexact_and_encloses(cuda_lib, oracle, shape):
    m, n, k = shape
    rng = np.random.default_rng(sum(shape) * 3)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -30)
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_PLAIN)
    assert np.array_equal(bits(C), bits(oracle.pidblas_mulmm(m, n, k, A, B)))
    rows = np.repeat(np.arange(m), n); cols = np.tile(np.arange(n), m)
    lo, up = oracle.exact_hull(m, n, k, A, B, rows, cols)
    idx = 2 * (rows + cols * m)
    assert np.all(C[idx] <= lo) and np.all(C[idx + 1] >= up)


def test_igemm_plain_golden(cuda_lib):
    g = np.load(GOLDEN)
    for idx in range(int(g["n_iv"][0])):
        m, n, k = map(int, g[f"iv{idx}_shape"])
        C = pidcuda.mulmm(g[f"iv{idx}_A"], g[f"iv{idx}_B"], m, n, k, form=pidcuda.FORM_PLAIN)
        assert np.array_equal(bits(C), bits(g[f"iv{idx}_C"])), idx


def test_igemm_plain_straddling_zero(cuda_lib, oracle):
    """Wide intervals that contain zero: every endpoint-product case."""
    rng = np.random.default_rng(13)
    m, n, k = 40, 30, 50
    A = W.interval_ephi(rng, m, k, 3, 1.5)
    B = W.interval_ephi(rng, k, n, 3, 0.9)
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_PLAIN)
    assert np.array_equal(bits(C), bits(oracle.pidblas_mulmm(m, n, k, A, B)))
    rows = np.repeat(np.arange(m), n); cols = np.tile(np.arange(n), m)
    lo, up = oracle.exact_hull(m, n, k, A, B, rows, cols)
    idx = 2 * (rows + cols * m)
    assert np.all(C[idx] <= lo) and np.all(C[idx + 1] >= up)


def test_igemm_dev_ld_and_stream(cuda_lib, oracle):
    import torch
    rng = np.random.default_rng(14)
    m, n, k = 70, 40, 90
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    ldc = 75
    dA = torch.from_numpy(A).cuda(); dB = torch.from_numpy(B).cuda()
    dC = torch.zeros(2 * ldc * n, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        pidcuda.mulmm_dev(m, n, k, dA, m, dB, k, dC, ldc, pidcuda.FORM_PLAIN, stream=s)
    s.synchronize()
    C = dC.cpu().numpy().reshape(n, ldc, 2)[:, :m, :].ravel()
    assert np.array_equal(bits(C), bits(oracle.pidblas_mulmm(m, n, k, A, B)))


def test_igemm_empty_inner(cuda_lib):
    C = pidcuda.mulmm(np.zeros(0), np.zeros(0), 3, 2, 0, form=pidcuda.FORM_PLAIN)
    assert np.all(C == 0.0)
    # lower ends are RD(0 - 0) = -0.0 as in pidblas (lC -= temp under round-down)
    assert np.all(np.signbit(C[0::2])) and not np.any(np.signbit(C[1::2]))
