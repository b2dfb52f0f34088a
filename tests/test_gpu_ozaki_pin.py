"""Parity of the tensor-core interval product at the sizes that are measured.

Every entry of the CRT form depends only on its row of A, its column of B
and the inner dimension (the per-row / per-column exponents, digit sums and
the modulus plan are functions of those alone), so the host model
(oracle/ozaki_model.c) run on a few full rows of A against all of B -- or on
all of A against a few full columns of B -- gives exactly the bits the GPU
must produce for those rows / columns of the full product.  That makes a
bit-for-bit check of the n = 8192 product (the headline configuration:
midpoints E(4), radius 2^-40 |mid|) affordable: O(k) model work per entry.

* n = 8192, device-resident form and host-pointer (blocked, overlapped)
  form: 16 full rows and 16 full columns bit-identical to the model, the two
  forms bit-identical to each other on those entries, and containment of the
  exact hull on sampled entries.
* k = 16384 (sixteen moduli, the largest plan at the default 56-bit
  operands) and k = 65536 (operands narrowed to keep sixteen moduli): every
  entry bit-identical to the model, and enclosing.
* Widths against the plain FP64 form for phi in {0, 8, 32}, radius ratios
  {0, 2^-40, 2^-20} and k in {2048, 8192} at the default 8 slices: never
  wider where the operands' digits resolve the plain form's rounding (the
  cases marked "not wider"); within a factor 2 everywhere (the bound on
  enclosure widths of the tensor-core form).  The tolerance is 0 ulp in the
  bit-exact tests.
"""
import numpy as np
import pytest

from vcp_gb300 import pidcuda
from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def rows_of(A, m, k, R):
    """kv buffer of rows R of the m x k column-major interval matrix A."""
    return np.ascontiguousarray(A.reshape(k, m, 2)[:, R, :]).ravel()


def cols_of(B, k, n, Cc):
    """kv buffer of columns Cc of the k x n column-major interval matrix B."""
    return np.ascontiguousarray(B.reshape(n, k, 2)[Cc]).ravel()


def block_of(C, m, n, R, Cc):
    """kv buffer (len(R) x len(Cc), column-major) of rows R, columns Cc of C."""
    return np.ascontiguousarray(C.reshape(n, m, 2)[np.ix_(Cc, R)]).ravel()


@pytest.fixture(scope="module")
def n8192_product(cuda_lib):
    import torch
    n = 8192
    rng = np.random.default_rng(8192)
    A = W.interval_ephi(rng, n, n, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, n, n, 4, 2.0 ** -40)
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    dC = torch.empty(2 * n * n, dtype=torch.float64, device="cuda")
    pidcuda.mulmm_dev(n, n, n, dA, n, dB, n, dC, n, pidcuda.FORM_OZAKI, 0)
    torch.cuda.synchronize()
    C_dev = dC.cpu().numpy()
    del dA, dB, dC
    torch.cuda.empty_cache()
    C_host = pidcuda.mulmm(A, B, n, n, n, form=pidcuda.FORM_OZAKI)
    return n, A, B, C_dev, C_host


def test_n8192_full_rows_bitexact_model(oracle, n8192_product):
    n, A, B, C_dev, C_host = n8192_product
    R = np.sort(np.random.default_rng(1).choice(n, 16, replace=False))
    R[0] = 0
    R[-1] = n - 1
    ref, st = oracle.ozaki_igemm(len(R), n, n, rows_of(A, n, n, R), B, 8, 2, crt=True)
    assert st == 0
    allc = np.arange(n)
    got_dev = block_of(C_dev, n, n, R, allc)
    got_host = block_of(C_host, n, n, R, allc)
    assert np.array_equal(bits(got_dev), bits(ref)), \
        f"{int(np.sum(bits(got_dev) != bits(ref)))} words differ from the model (device form)"
    assert np.array_equal(bits(got_host), bits(ref)), "host-pointer form differs from the model"


def test_n8192_full_columns_bitexact_model(oracle, n8192_product):
    n, A, B, C_dev, C_host = n8192_product
    Cc = np.sort(np.random.default_rng(2).choice(n, 16, replace=False))
    Cc[0] = 0
    Cc[-1] = n - 1
    ref, st = oracle.ozaki_igemm(n, len(Cc), n, A, cols_of(B, n, n, Cc), 8, 2, crt=True)
    assert st == 0
    allr = np.arange(n)
    assert np.array_equal(bits(block_of(C_dev, n, n, allr, Cc)), bits(ref))
    assert np.array_equal(bits(block_of(C_host, n, n, allr, Cc)), bits(ref))


def test_n8192_sampled_containment(oracle, n8192_product):
    n, A, B, C_dev, _ = n8192_product
    rng = np.random.default_rng(3)
    rows = rng.integers(0, n, 1024).astype(np.int32)
    cols = rng.integers(0, n, 1024).astype(np.int32)
    lo, up = oracle.exact_hull(n, n, n, A, B, rows, cols)
    idx = 2 * (rows.astype(np.int64) + cols.astype(np.int64) * n)
    assert np.all(C_dev[idx] <= lo) and np.all(C_dev[idx + 1] >= up)


@pytest.mark.parametrize("m,n,k", [(200, 190, 16384), (64, 72, 65536)])
def test_long_inner_dimension_bitexact_model(cuda_lib, oracle, m, n, k):
    rng = np.random.default_rng(k)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI)
    ref, st = oracle.ozaki_igemm(m, n, k, A, B, 8, 2, crt=True)
    assert st == 0
    assert np.array_equal(bits(C), bits(ref))
    rows = np.repeat(np.arange(m), n)[::7].astype(np.int32)
    cols = np.tile(np.arange(n), m)[::7].astype(np.int32)
    lo, up = oracle.exact_hull(m, n, k, A, B, rows, cols)
    idx = 2 * (rows.astype(np.int64) + cols.astype(np.int64) * m)
    assert np.all(C[idx] <= lo) and np.all(C[idx + 1] >= up)


# (k, phi, radius ratio) -> the default 8 slices are never wider than the
# plain form there.  Elsewhere the digits of the radius factors (16 bits
# relative to the row / column maximum) or the 2^-56 operand truncation at
# a 2^64 exponent spread can exceed the plain form's own rounding by a few
# percent; those cases are bounded by the factor 2.  NOT_WIDER_FAST: the
# same with the fast radius products (the bound of their left-out low x low
# digit pair adds up to 3 % at the 2^64 spread).
NOT_WIDER = {(2048, 0, 0.0), (2048, 0, 2.0 ** -40), (2048, 8, 0.0), (2048, 8, 2.0 ** -40),
             (8192, 0, 0.0), (8192, 0, 2.0 ** -40), (8192, 8, 0.0), (8192, 8, 2.0 ** -40),
             (8192, 32, 0.0), (8192, 32, 2.0 ** -40)}
NOT_WIDER_FAST = NOT_WIDER - {(8192, 32, 2.0 ** -40)}


@pytest.mark.parametrize("k", [2048, 8192])
@pytest.mark.parametrize("phi", [0, 8, 32])
@pytest.mark.parametrize("rr", [0.0, 2.0 ** -40, 2.0 ** -20], ids=["r0", "r2e-40", "r2e-20"])
def test_width_against_plain(cuda_lib, k, phi, rr):
    rng = np.random.default_rng(1000 * phi + k + (rr > 0) + (rr > 1e-9))
    m = n = 256
    A = W.interval_ephi(rng, m, k, phi, rr)
    B = W.interval_ephi(rng, k, n, phi, rr)
    Co = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI)
    Cp = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_PLAIN)
    wo = Co[1::2] - Co[0::2]
    wp = Cp[1::2] - Cp[0::2]
    ratio = wo / wp
    assert np.all(np.isfinite(ratio))
    assert np.max(ratio) <= 2.0, float(np.max(ratio))
    if (k, phi, rr) in NOT_WIDER:
        assert np.all(wo <= wp), float(np.max(ratio))
    Cf = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI,
                       slices=8 | pidcuda.SLICES_FAST_RADIUS)
    wf = Cf[1::2] - Cf[0::2]
    assert np.max(wf / wp) <= 2.0, float(np.max(wf / wp))
    assert np.all(wf >= wo)  # the bound of the left-out pair only adds
    if (k, phi, rr) in NOT_WIDER_FAST:
        assert np.all(wf <= wp), float(np.max(wf / wp))
