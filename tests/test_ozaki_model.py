"""CPU tests of the host model of the tensor-core (CRT) form: its
enclosures contain the exact interval hull, with the exact radius products
(the default) and with the fast ones (slices + 0x100), including the cases
where the fast products' left-out pair of low digits is as large as it can
be -- every low digit 127 on both sides, so that sum_k lo_A lo_B reaches
the Cauchy-Schwarz bound the reassembly adds for it (a model without that
term fails these cases: the radius would lose 127^2 / 25727^2 of its size)
-- and that the enclosures stay no wider than the plain form's at the
benchmark distribution."""
import numpy as np
import pytest

from vcp_gb300 import workloads as W

# 25727 2^-16 = 0.39256..., the 16-bit radius digits (100, 127) against a
# row / column maximum of itself
X_LOW127 = 25727 * 2.0 ** -16
FAST = 0x100  # the fast-radius flag of the slices argument


def _kv(mid, rad):
    out = np.empty(2 * mid.size)
    out[0::2] = mid - rad
    out[1::2] = mid + rad
    return out


def _contains(oracle, m, n, k, A, B, C):
    rows = np.repeat(np.arange(m), n)
    cols = np.tile(np.arange(n), m)
    lo, up = oracle.exact_hull(m, n, k, A, B, rows, cols)
    idx = 2 * (rows + cols * m)
    return bool(np.all(C[idx] <= lo) and np.all(C[idx + 1] >= up))


def low127_operands(side, m, n, k, seed=3):
    """side 0: the product (|mA| + rA) rB with every low digit 127 (A a point
    matrix of X_LOW127, rB = X_LOW127 2^-30); side 1: rA |mB| (B a point
    matrix of X_LOW127, rA = X_LOW127 2^-30)."""
    rng = np.random.default_rng(seed)
    r = X_LOW127 * 2.0 ** -30
    if side == 0:
        A = _kv(np.full(m * k, X_LOW127), np.zeros(m * k))
        B = _kv(rng.uniform(0.5, 1.0, k * n), np.full(k * n, r))
    else:
        A = _kv(rng.uniform(0.5, 1.0, m * k), np.full(m * k, r))
        B = _kv(np.full(k * n, X_LOW127), np.zeros(k * n))
    return A, B


@pytest.mark.parametrize("s", [8 | FAST, 8], ids=["fast", "exact"])
def test_model_low_pair_bound_left(oracle, s):
    m, n, k = 24, 20, 3000
    A, B = low127_operands(0, m, n, k)
    C, st = oracle.ozaki_igemm(m, n, k, A, B, s, 2)
    assert st == 0
    assert _contains(oracle, m, n, k, A, B, C)


@pytest.mark.parametrize("s", [8 | FAST, 8], ids=["fast", "exact"])
def test_model_low_pair_bound_right(oracle, s):
    m, n, k = 20, 24, 2100
    A, B = low127_operands(1, m, n, k)
    C, st = oracle.ozaki_igemm(m, n, k, A, B, s, 2)
    assert st == 0
    assert _contains(oracle, m, n, k, A, B, C)


def test_model_encloses_and_not_wider(oracle):
    rng = np.random.default_rng(9)
    m, n, k = 40, 36, 1500
    for A, B in [(W.interval_uniform(rng, m, k, 1e-12), W.interval_uniform(rng, k, n, 1e-12)),
                 (W.interval_ephi(rng, m, k, 4, 2.0 ** -40),
                  W.interval_ephi(rng, k, n, 4, 2.0 ** -40))]:
        P = oracle.pidblas_mulmm(m, n, k, A, B)
        for s in (8, 8 | FAST):
            C, st = oracle.ozaki_igemm(m, n, k, A, B, s, 2)
            assert st == 0
            assert _contains(oracle, m, n, k, A, B, C)
            assert np.all(C[1::2] - C[0::2] <= P[1::2] - P[0::2])


def test_model_slice_form_encloses(oracle):
    """The slice form keeps all four radius digit pairs (no bound term)."""
    m, n, k = 24, 20, 3000
    A, B = low127_operands(0, m, n, k)
    C, st = oracle.ozaki_igemm(m, n, k, A, B, 8, 2, crt=False)
    assert st == 0
    assert _contains(oracle, m, n, k, A, B, C)
