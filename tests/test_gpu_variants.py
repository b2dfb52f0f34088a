"""GPU parity of the other products on the path, through the C ABI:
interval x point (pidblas::mul_im_m / mul_m_im), [A]^T[A] (pidblas::mulltmm),
verified A^T A (pidblas::vmulmm) and the ||R[A] - I||_inf bound of
imats::linearsolve.  Plain form: bit-identical to the oracle (pinned to the
reference).  Ozaki forms: enclose the exact hull (long accumulator)."""
from pathlib import Path

import numpy as np
import pytest

from vcp_gb300 import pidcuda
from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def degenerate(P):
    out = np.empty(2 * P.size)
    out[0::2] = P
    out[1::2] = P
    return out


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("shape", [(1, 1, 1), (33, 65, 70), (130, 20, 300), (7, 200, 17)])
def test_mul_point_plain_bitexact_and_ozaki_encloses(cuda_lib, oracle, side, shape):
    m, n, k = shape
    rng = np.random.default_rng(side * 1000 + sum(shape))
    L = W.interval_ephi(rng, m, k, 4, 2.0 ** -30) if side == 0 else W.ephi(rng, m * k, 4)
    R = W.ephi(rng, k * n, 4) if side == 0 else W.interval_ephi(rng, k, n, 4, 2.0 ** -30)
    C = pidcuda.mul_point(side, L, R, m, n, k, form=pidcuda.FORM_PLAIN)
    assert np.array_equal(bits(C), bits(oracle.pidblas_mul_point(side, m, n, k, L, R)))
    Li = L if side == 0 else degenerate(L)
    Ri = degenerate(R) if side == 0 else R
    rows = np.repeat(np.arange(m), n)
    cols = np.tile(np.arange(n), m)
    lo, up = oracle.exact_hull(m, n, k, Li, Ri, rows, cols)
    idx = 2 * (rows + cols * m)
    for form in (pidcuda.FORM_OZAKI, pidcuda.FORM_OZAKI_SLICES):
        Co = pidcuda.mul_point(side, L, R, m, n, k, form=form)
        assert np.all(Co[idx] <= lo) and np.all(Co[idx + 1] >= up)
        # the GPU skips the radius product with the zero factor; the host
        # model runs both on the degenerate operands: same bits
        Cm, _ = oracle.ozaki_igemm(m, n, k, Li, Ri, crt=form == pidcuda.FORM_OZAKI)
        assert np.array_equal(bits(Co), bits(Cm)), form


def test_other_products_golden(cuda_lib):
    g = np.load(GOLDEN)
    for idx in range(int(g["n_mp"][0])):
        side, m, n, k = map(int, g[f"mp{idx}_shape"])
        C = pidcuda.mul_point(side, g[f"mp{idx}_L"], g[f"mp{idx}_R"], m, n, k)
        assert np.array_equal(bits(C), bits(g[f"mp{idx}_C"])), idx
    for idx in range(int(g["n_sy"][0])):
        n, k = map(int, g[f"sy{idx}_shape"])
        assert np.array_equal(bits(pidcuda.isyrk(g[f"sy{idx}_A"], n, k)), bits(g[f"sy{idx}_C"]))
        assert np.array_equal(bits(pidcuda.vsyrk(g[f"sy{idx}_P"], n, k)), bits(g[f"sy{idx}_V"]))
    for idx in range(int(g["n_nm"][0])):
        n = int(g[f"nm{idx}_n"][0])
        assert pidcuda.norm_I_minus_RA(g[f"nm{idx}_R"], g[f"nm{idx}_A"], n) == \
            float(g[f"nm{idx}_bound"][0])


@pytest.mark.parametrize("shape", [(1, 1), (20, 7), (65, 130), (130, 64), (200, 33)])
def test_isyrk_vsyrk(cuda_lib, oracle, shape):
    n, k = shape
    rng = np.random.default_rng(n * 31 + k)
    A = W.interval_ephi(rng, k, n, 4, 2.0 ** -25)
    C = pidcuda.isyrk(A, n, k)
    assert np.array_equal(bits(C), bits(oracle.pidblas_mulltmm(n, k, A)))
    P = W.ephi(rng, k * n, 8)
    V = pidcuda.vsyrk(P, n, k)
    assert np.array_equal(bits(V), bits(oracle.pidblas_vmulmm(n, k, P)))
    # Ozaki forms enclose the exact hull of [A]^T [A]
    At = A.reshape(n, k, 2).transpose(1, 0, 2).copy().reshape(-1)  # (n x k) interval
    rows = np.repeat(np.arange(n), n)
    cols = np.tile(np.arange(n), n)
    lo, up = oracle.exact_hull(n, n, k, At, A, rows, cols)
    idx = 2 * (rows + cols * n)
    for form in (pidcuda.FORM_OZAKI, pidcuda.FORM_OZAKI_SLICES):
        Co = pidcuda.isyrk(A, n, k, form=form)
        assert np.all(Co[idx] <= lo) and np.all(Co[idx + 1] >= up)


@pytest.mark.parametrize("n", [1, 50, 257])
def test_norm_bound(cuda_lib, oracle, n):
    rng = np.random.default_rng(n)
    Am = np.eye(n) + 0.1 * rng.standard_normal((n, n)) / np.sqrt(n)
    Ai = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * 1e-8)
    Rinv = np.linalg.inv(Am).ravel(order="F")
    g = pidcuda.norm_I_minus_RA(Rinv, Ai, n)
    assert g == oracle.norm_I_minus_RA(n, Rinv, Ai)
    assert 0 <= g < 1
    # every form bounds the norm over the exact hull of R [A] from above
    Ri = degenerate(Rinv)
    rows = np.repeat(np.arange(n), n)
    cols = np.tile(np.arange(n), n)
    lo, up = oracle.exact_hull(n, n, n, Ri, Ai, rows, cols)
    d = (rows == cols).astype(float)
    mag = np.maximum(np.abs(lo - d), np.abs(up - d)).reshape(n, n)
    approx = float(np.max(mag.sum(axis=1)))
    for form in (pidcuda.FORM_OZAKI, pidcuda.FORM_OZAKI_SLICES):
        go = pidcuda.norm_I_minus_RA(Rinv, Ai, n, form=form)
        assert approx * (1 - 1e-9) <= go < 1
    assert approx * (1 - 1e-9) <= g
