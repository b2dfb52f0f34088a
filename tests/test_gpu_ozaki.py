"""GPU parity of the Ozaki (tensor-core) forms of the interval product.

* FORM_OZAKI (CRT form) is bit-identical to the host model
  oracle/ozaki_model.c, which computes the exact product of the w-bit
  integer operands directly in 128-bit integers -- so equality also proves
  the residue GEMMs and the Chinese remaindering exact; FORM_OZAKI_SLICES
  (triangular digit slices) is bit-identical to the slice host model (same
  slicing, summation order, folds and directed reassembly).  Cases: ragged
  shapes, several precisions, inner dimensions spanning several
  1024-element chunks, and extreme digit patterns (chunk sums of +-2^24);
* zero containment failures against the exact interval hull (long
  accumulator) on every checked entry;
* with SLICES_FAST_RADIUS the CRT form's radius products leave out the pair
  of the two low digits and the reassembly adds its Cauchy-Schwarz bound:
  bit-identical to the model and enclosing where every low digit is 127
  (the bound is tight);
* enclosure no wider than the plain FP64 form at the benchmark distribution;
* non-finite inputs give NaN results and VCPCU_ERR_NONFINITE.
"""
import numpy as np
import pytest

from vcp_gb300 import pidcuda
from vcp_gb300 import workloads as W
from vcp_gb300.errors import NonFiniteError

pytestmark = pytest.mark.gpu


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def check_contains(oracle, m, n, k, A, B, C, rows=None, cols=None):
    if rows is None:
        rows = np.repeat(np.arange(m), n)
        cols = np.tile(np.arange(n), m)
    lo, up = oracle.exact_hull(m, n, k, A, B, rows, cols)
    idx = 2 * (rows + cols * m)
    assert np.all(C[idx] <= lo), "lower end above the exact hull"
    assert np.all(C[idx + 1] >= up), "upper end below the exact hull"


CASES = [(1, 1, 1, 8), (5, 7, 3, 8), (128, 256, 64, 8), (129, 257, 65, 6), (200, 100, 1500, 8),
         (64, 300, 2048, 4), (33, 40, 999, 12), (256, 256, 256, 2)]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("crt", [True, False, "fast"], ids=["crt", "slices", "crt-fast-radius"])
def test_ozaki_bitexact_model_and_encloses(cuda_lib, oracle, case, crt):
    m, n, k, s = case
    rng = np.random.default_rng(m * 7 + n * 3 + k + s)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    form = pidcuda.FORM_OZAKI if crt else pidcuda.FORM_OZAKI_SLICES
    if crt == "fast":  # the low x low radius pair left out and bounded
        s |= pidcuda.SLICES_FAST_RADIUS
    C = pidcuda.mulmm(A, B, m, n, k, form=form, slices=s)
    ref, st = oracle.ozaki_igemm(m, n, k, A, B, s, 2, crt=bool(crt))
    assert st == 0
    assert np.array_equal(bits(C), bits(ref)), "GPU differs from the host model"
    check_contains(oracle, m, n, k, A, B, C)


@pytest.mark.parametrize("k", [3000, 8192])
def test_ozaki_extreme_digits(cuda_lib, oracle, k):
    """All midpoints equal in magnitude: every top digit is +-128 and every
    1024-chunk of digit products sums to +-2^24, the exactness limit -- at
    k = 8192 (the bench's inner dimension) eight full chunks per entry."""
    m, n = 130, 260
    A = np.empty(2 * m * k); B = np.empty(2 * k * n)
    A[0::2] = A[1::2] = 1.0
    B[0::2] = B[1::2] = 1.0
    for form, crt in ((pidcuda.FORM_OZAKI, True), (pidcuda.FORM_OZAKI_SLICES, False)):
        C = pidcuda.mulmm(A, B, m, n, k, form=form, slices=8)
        ref, _ = oracle.ozaki_igemm(m, n, k, A, B, 8, 2, crt=crt)
        assert np.array_equal(bits(C), bits(ref))
        assert np.all(C[0::2] <= k) and np.all(C[1::2] >= k)
    # alternating signs by column of A: cancellation to exactly zero
    rng = np.random.default_rng(2)
    sg = np.where(rng.random(m * k) < 0.5, -1.0, 1.0)
    A[0::2] = A[1::2] = sg
    for form, crt in ((pidcuda.FORM_OZAKI, True), (pidcuda.FORM_OZAKI_SLICES, False)):
        C = pidcuda.mulmm(A, B, m, n, k, form=form, slices=8)
        ref, _ = oracle.ozaki_igemm(m, n, k, A, B, 8, 2, crt=crt)
        assert np.array_equal(bits(C), bits(ref))
    check_contains(oracle, m, n, k, A, B, C, rows=np.arange(0, m, 7).repeat(4),
                   cols=np.tile(np.array([0, 1, 100, 259]), len(range(0, m, 7))))


def test_ozaki_wide_and_straddling(cuda_lib, oracle):
    rng = np.random.default_rng(3)
    m, n, k = 90, 70, 500
    A = W.interval_ephi(rng, m, k, 20, 0.9)
    B = W.interval_ephi(rng, k, n, 20, 1.7)
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI, slices=5)
    ref, _ = oracle.ozaki_igemm(m, n, k, A, B, 5, 2)
    assert np.array_equal(bits(C), bits(ref))
    check_contains(oracle, m, n, k, A, B, C)


def test_ozaki_zero_rows_and_columns(cuda_lib, oracle):
    rng = np.random.default_rng(4)
    m, n, k = 40, 50, 300
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    A.reshape(k, m, 2)[:, 3, :] = 0.0     # row 3 of A is [0, 0]
    B.reshape(n, k, 2)[7, :, :] = 0.0     # column 7 of B is [0, 0]
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI, slices=8)
    ref, _ = oracle.ozaki_igemm(m, n, k, A, B, 8, 2)
    assert np.array_equal(bits(C), bits(ref))
    check_contains(oracle, m, n, k, A, B, C)


@pytest.mark.parametrize("fast", [pidcuda.SLICES_FAST_RADIUS, 0], ids=["bound", "exact"])
@pytest.mark.parametrize("side", [0, 1])
def test_ozaki_low_pair_bound(cuda_lib, oracle, side, fast):
    from test_ozaki_model import low127_operands
    m, n, k = (24, 20, 3000) if side == 0 else (20, 24, 2100)
    A, B = low127_operands(side, m, n, k)
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI, slices=8 | fast)
    ref, st = oracle.ozaki_igemm(m, n, k, A, B, 8 | fast, 2)
    assert st == 0 and np.array_equal(bits(C), bits(ref))
    check_contains(oracle, m, n, k, A, B, C)


def test_ozaki_not_wider_than_plain(cuda_lib):
    """At the benchmark distribution (mid E(4), rad 2^-40 |mid|) and k = 2048
    the default 8 slices give enclosures no wider than the plain form."""
    rng = np.random.default_rng(5)
    m = n = 256
    k = 2048
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    Co = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI, slices=8)
    Cp = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_PLAIN)
    wo = Co[1::2] - Co[0::2]
    wp = Cp[1::2] - Cp[0::2]
    assert np.all(wo <= wp), float(np.max(wo / wp))


def test_ozaki_nonfinite(cuda_lib):
    rng = np.random.default_rng(6)
    m, n, k = 20, 20, 30
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    A[10] = np.inf
    C = np.zeros(2 * m * n)
    with pytest.raises(NonFiniteError):
        pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI, out=C)
    assert np.all(np.isnan(C))
    # the sticky status is cleared: the next call is clean
    A[10] = 1.0
    pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI)


def test_ozaki_dev_stream(cuda_lib, oracle):
    import torch
    rng = np.random.default_rng(7)
    m, n, k = 150, 140, 700
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    ldc = 160
    dA = torch.from_numpy(A).cuda(); dB = torch.from_numpy(B).cuda()
    dC = torch.zeros(2 * ldc * n, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    pidcuda.mulmm_dev(m, n, k, dA, m, dB, k, dC, ldc, pidcuda.FORM_OZAKI, 7, stream=s)
    from vcp_gb300 import _lib
    _lib.call("vcpcu_status", s.cuda_stream)
    C = dC.cpu().numpy().reshape(n, ldc, 2)[:, :m, :].ravel()
    ref, _ = oracle.ozaki_igemm(m, n, k, A, B, 7, 2)
    assert np.array_equal(bits(C), bits(ref))


def mixed_intervals(rng, rows, cols):
    """Entries that take every branch of the operand preparation: narrow
    intervals of either sign (the integer-pipe midrad), adjacent doubles
    (rounding ties of the midpoint), intervals straddling zero, wide ones,
    degenerate ones, subnormal and near-overflow endpoints, signed zeros."""
    n = rows * cols
    kind = rng.integers(0, 9, n)
    mid = W.ephi(rng, n, 6)
    lo = mid - np.abs(mid) * 2.0 ** -40
    up = mid + np.abs(mid) * 2.0 ** -40
    adj = kind == 1
    lo[adj] = mid[adj]
    up[adj] = np.nextafter(mid[adj], np.inf)
    st = kind == 2
    lo[st] = -np.abs(mid[st]) * 0.3
    up[st] = np.abs(mid[st])
    wide = kind == 3
    lo[wide] = np.abs(mid[wide]) * 0.1
    up[wide] = np.abs(mid[wide]) * 7.0
    deg = kind == 4
    lo[deg] = up[deg] = mid[deg]
    sub = kind == 5
    lo[sub] = 3e-310
    up[sub] = 5e-310
    big = kind == 6
    lo[big] = np.abs(mid[big]) * 1e290
    up[big] = np.nextafter(lo[big], np.inf)
    zer = kind == 7
    lo[zer] = -0.0
    up[zer] = 0.0
    ulps = kind == 8
    lo[ulps] = mid[ulps]
    up[ulps] = mid[ulps] + np.abs(mid[ulps]) * 2.0 ** -50
    out = np.empty(2 * n)
    out[0::2], out[1::2] = np.minimum(lo, up), np.maximum(lo, up)
    return out


@pytest.mark.parametrize("crt", [True, False], ids=["crt", "slices"])
def test_ozaki_midrad_paths(cuda_lib, oracle, crt):
    """Bit-identical to the host model (FP64 midrad) on entries that take the
    integer-pipe midrad and every fall-back to the FP64 instructions."""
    rng = np.random.default_rng(17)
    m, n, k = 70, 60, 400
    A = mixed_intervals(rng, m, k)
    B = mixed_intervals(rng, k, n)
    B[0::2] *= 1e-300   # keep the products of the near-overflow rows finite
    B[1::2] *= 1e-300
    form = pidcuda.FORM_OZAKI if crt else pidcuda.FORM_OZAKI_SLICES
    C = pidcuda.mulmm(A, B, m, n, k, form=form, slices=8)
    ref, st = oracle.ozaki_igemm(m, n, k, A, B, 8, 2, crt=crt)
    assert st == 0
    assert np.array_equal(bits(C), bits(ref))
    check_contains(oracle, m, n, k, A, B, C)


@pytest.mark.parametrize("shape,panels,row_panels", [
    ((300, 2048, 500), None, None), ((129, 700, 1100), "2", "2"), ((64, 1300, 70), "5", "1"),
    ((33, 600, 0), "3", "2"), ((700, 900, 300), "2", "3"), ((4096, 256, 64), "1", "4")])
def test_ozaki_host_pipeline_bitexact(cuda_lib, shape, panels, row_panels, monkeypatch):
    """The host-pointer call overlaps its copies with blocks of the product
    (row blocks of A, column blocks of B, interleaved uploads, each block of
    C sent down when done); the result is bit-identical to the one-shot
    device call, including last blocks of smaller padded size, a row block
    of one row and an empty inner dimension."""
    import torch
    from vcp_gb300 import _lib
    m, n, k = shape
    if panels is not None:
        monkeypatch.setenv("VCPCU_HOST_PANELS", panels)
    if row_panels is not None:
        monkeypatch.setenv("VCPCU_HOST_ROW_PANELS", row_panels)
    rng = np.random.default_rng(m + n + k)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40) if k else np.zeros(0)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40) if k else np.zeros(0)
    hA = torch.from_numpy(A).pin_memory() if k else torch.zeros(2, dtype=torch.float64)
    hB = torch.from_numpy(B).pin_memory() if k else torch.zeros(2, dtype=torch.float64)
    hC = torch.full((2 * m * n,), 7.0, dtype=torch.float64).pin_memory()
    _lib.call("vcpcu_igemm", m, n, k, hA.data_ptr(), hB.data_ptr(), hC.data_ptr(),
              pidcuda.FORM_OZAKI, 0)
    dA = hA.cuda(); dB = hB.cuda()
    dC = torch.zeros(2 * m * n, dtype=torch.float64, device="cuda")
    pidcuda.mulmm_dev(m, n, k, dA, m, dB, max(k, 1), dC, m, pidcuda.FORM_OZAKI, 0)
    _lib.call("vcpcu_status", 0)
    assert np.array_equal(bits(hC.numpy()), bits(dC.cpu().numpy()))


def test_ozaki_host_pipeline_nonfinite_late_panel(cuda_lib, monkeypatch):
    """A non-finite entry in the last column panel of B still makes every
    entry NaN (earlier panels were already copied back finite)."""
    import torch
    from vcp_gb300 import _lib
    monkeypatch.setenv("VCPCU_HOST_PANELS", "4")
    m, n, k = 40, 1024, 50
    rng = np.random.default_rng(11)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    B[2 * (5 + (n - 1) * k) + 1] = np.inf
    hA = torch.from_numpy(A).pin_memory()
    hB = torch.from_numpy(B).pin_memory()
    hC = torch.zeros(2 * m * n, dtype=torch.float64).pin_memory()
    with pytest.raises(NonFiniteError):
        _lib.call("vcpcu_igemm", m, n, k, hA.data_ptr(), hB.data_ptr(), hC.data_ptr(),
                  pidcuda.FORM_OZAKI, 0)
    assert np.all(np.isnan(hC.numpy()))


def test_ozaki_host_pipeline_pageable(cuda_lib):
    """The blocked host-pointer path with ordinary (pageable) numpy buffers:
    the copies are staged, the result is the same bits as the device call."""
    import torch
    from vcp_gb300 import _lib
    m, n, k = 300, 2300, 700
    rng = np.random.default_rng(33)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI)
    dA = torch.from_numpy(A).cuda(); dB = torch.from_numpy(B).cuda()
    dC = torch.zeros(2 * m * n, dtype=torch.float64, device="cuda")
    pidcuda.mulmm_dev(m, n, k, dA, m, dB, k, dC, m, pidcuda.FORM_OZAKI, 0)
    _lib.call("vcpcu_status", 0)
    assert np.array_equal(bits(C), bits(dC.cpu().numpy()))
