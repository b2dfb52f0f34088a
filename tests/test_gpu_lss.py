"""GPU parity of the verified linear solve's device-resident part
(vcpcu_ilss_verify: imats::linearsolve, vcp/imats.hpp:293-364, after R and
mx) and of the thin plain kernel its matrix-vector products run on.

* Plain form: every bit of x and the bound equal the reference's
  (golden vectors from the reference's own linearsolve) and the oracle's
  restatement (pinned to the reference) on random systems.
* Tensor-core form: bit-identical to the restatement fed with the GPU's
  own R[A] (itself bit-identical to the host model), and the enclosures
  hold the exact rational solutions of integer systems.
"""
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from vcp_gb300 import pidcuda
from vcp_gb300 import workloads as W
from vcp_gb300.errors import VerificationError

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def mid_of(X):
    """kv midpoints (numpy, nearest): only an approximation for R and mx."""
    return 0.5 * (X[0::2] + X[1::2])


def system(rng, n, nrhs, rel, shift=4.0):
    Am = rng.uniform(-1.0, 1.0, (n, n)) + shift * np.eye(n)
    A = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * rel)
    bm = rng.uniform(-1.0, 1.0, n * nrhs)
    b = W._kv(bm, np.abs(bm) * 2.0 ** -35)
    R = np.linalg.inv(mid_of(A).reshape(n, n, order="F"))
    mx = R @ mid_of(b).reshape(n, nrhs, order="F")
    return A, b, R.ravel(order="F").copy(), mx.ravel(order="F").copy()


def rational_solve(M, b):
    n = len(M)
    cols = b.shape[1]
    a = [[Fraction(int(M[i, j])) for j in range(n)] + [Fraction(int(b[i, c])) for c in range(cols)]
         for i in range(n)]
    for c in range(n):
        p = next(r for r in range(c, n) if a[r][c] != 0)
        a[c], a[p] = a[p], a[c]
        for r in range(n):
            if r != c and a[r][c] != 0:
                f = a[r][c] / a[c][c]
                a[r] = [x - f * y for x, y in zip(a[r], a[c])]
    return [[a[i][n + c] / a[i][i] for c in range(cols)] for i in range(n)]


# ---- the thin plain kernel ---------------------------------------------------

@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 9, 16])
@pytest.mark.parametrize("mk", [(1, 1), (31, 63), (257, 130), (40, 0)])
def test_thin_plain_bitexact(cuda_lib, oracle, n, mk):
    m, k = mk
    rng = np.random.default_rng(100 * n + m + k)
    A = W.interval_ephi(rng, m, max(k, 1), 6, 2.0 ** -20)[: 2 * m * k]
    B = W.interval_ephi(rng, max(k, 1), n, 6, 2.0 ** -10)[: 2 * k * n]
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_PLAIN)
    assert np.array_equal(bits(C), bits(oracle.pidblas_mulmm(m, n, k, A, B)))


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("n", [1, 4, 13])
def test_thin_point_sides_bitexact(cuda_lib, oracle, side, n):
    m, k = 77, 190
    rng = np.random.default_rng(7 * n + side)
    L = W.interval_ephi(rng, m, k, 4, 2.0 ** -30) if side == 0 else W.ephi(rng, m * k, 4)
    R = W.ephi(rng, k * n, 4) if side == 0 else W.interval_ephi(rng, k, n, 4, 2.0 ** -30)
    C = pidcuda.mul_point(side, L, R, m, n, k, form=pidcuda.FORM_PLAIN)
    assert np.array_equal(bits(C), bits(oracle.pidblas_mul_point(side, m, n, k, L, R)))


# ---- the verification chain --------------------------------------------------

def test_ilss_plain_matches_reference_golden(cuda_lib):
    g = np.load(GOLDEN)
    for idx in range(int(g["n_ls"][0])):
        n, nrhs = map(int, g[f"ls{idx}_shape"])
        args = (g[f"ls{idx}_A"], g[f"ls{idx}_b"], g[f"ls{idx}_R"], g[f"ls{idx}_mx"], n, nrhs)
        x, G = pidcuda.linearsolve_verify(*args, form=pidcuda.FORM_PLAIN, check=False)
        assert G == float(g[f"ls{idx}_bound"][0]), idx
        if int(g[f"ls{idx}_status"][0]) == 0:
            assert np.array_equal(bits(x), bits(g[f"ls{idx}_x"])), idx
        else:
            with pytest.raises(VerificationError):
                pidcuda.linearsolve_verify(*args, form=pidcuda.FORM_PLAIN)


@pytest.mark.parametrize("shape", [(2, 1), (7, 2), (64, 1), (100, 4), (130, 7), (96, 16),
                                   (80, 20)])
def test_ilss_plain_matches_oracle(cuda_lib, oracle, shape):
    n, nrhs = shape
    rng = np.random.default_rng(n * 31 + nrhs)
    A, b, R, mx = system(rng, n, nrhs, 2.0 ** -30)
    x, G = pidcuda.linearsolve_verify(A, b, R, mx, n, nrhs, form=pidcuda.FORM_PLAIN)
    st, xo, Go = oracle.ilss_verify(n, nrhs, A, b, R, mx)
    assert st == 0 and G == Go
    assert np.array_equal(bits(x), bits(xo))


@pytest.mark.parametrize("shape", [(64, 1), (200, 3), (129, 4)])
def test_ilss_ozaki_matches_restatement(cuda_lib, oracle, shape):
    """The tensor-core R[A] (bit-identical to its host model elsewhere)
    fed to the restatement reproduces every bit of the chain."""
    n, nrhs = shape
    rng = np.random.default_rng(n + 17 * nrhs)
    A, b, R, mx = system(rng, n, nrhs, 2.0 ** -36)
    x, G = pidcuda.linearsolve_verify(A, b, R, mx, n, nrhs, form=pidcuda.FORM_OZAKI)
    E = pidcuda.mul_point(1, R, A, n, n, n, form=pidcuda.FORM_OZAKI)
    st, xo, Go = oracle.ilss_verify(n, nrhs, A, b, R, mx, E=E)
    assert st == 0 and G == Go
    assert np.array_equal(bits(x), bits(xo))
    xp, Gp = pidcuda.linearsolve_verify(A, b, R, mx, n, nrhs, form=pidcuda.FORM_PLAIN)
    # both enclose the solution set; widths within a few percent of each other
    wo, wp = x[1::2] - x[0::2], xp[1::2] - xp[0::2]
    assert np.median(wo / wp) < 1.05


@pytest.mark.parametrize("form", [pidcuda.FORM_PLAIN, pidcuda.FORM_OZAKI, pidcuda.FORM_AUTO])
@pytest.mark.parametrize("nrhs", [1, 3, 8])
def test_ilss_encloses_exact_solution(cuda_lib, form, nrhs):
    n = 24
    rng = np.random.default_rng(nrhs + 3 * form)
    M = np.round(rng.uniform(-9, 9, (n, n))) + 60 * np.eye(n)
    bb = np.round(rng.uniform(-9, 9, (n, nrhs)))
    A = W._kv(M.ravel(order="F"), np.zeros(n * n))
    b = W._kv(bb.ravel(order="F"), np.zeros(n * nrhs))
    R = np.linalg.inv(M).ravel(order="F").copy()
    mx = (R.reshape(n, n, order="F") @ bb).ravel(order="F").copy()
    x, G = pidcuda.linearsolve_verify(A, b, R, mx, n, nrhs, form=form)
    assert G < 1e-10
    exact = rational_solve(M, bb)
    for j in range(nrhs):
        for i in range(n):
            t = i + j * n
            assert Fraction(x[2 * t]) <= exact[i][j] <= Fraction(x[2 * t + 1]), (i, j)


def test_ilss_failed_check_raises(cuda_lib, oracle):
    n = 10
    rng = np.random.default_rng(3)
    A, b, R, mx = system(rng, n, 1, 0.5, shift=2.0)
    _, Go = pidcuda.linearsolve_verify(A, b, R, mx, n, 1, form=pidcuda.FORM_PLAIN, check=False)
    st, _, G = oracle.ilss_verify(n, 1, A, b, R, mx)
    assert st == 2 and Go == G and G >= 1.0
    with pytest.raises(VerificationError):
        pidcuda.linearsolve_verify(A, b, R, mx, n, 1, form=pidcuda.FORM_PLAIN)


@pytest.mark.parametrize("form", [pidcuda.FORM_PLAIN, pidcuda.FORM_OZAKI])
def test_ilss_device_form_matches_host_form(cuda_lib, form):
    import torch
    n, nrhs = 150, 2
    rng = np.random.default_rng(11 + form)
    A, b, R, mx = system(rng, n, nrhs, 2.0 ** -30)
    x, G = pidcuda.linearsolve_verify(A, b, R, mx, n, nrhs, form=form)
    dev = torch.device("cuda")
    tA, tb, tR, tm = (torch.from_numpy(v).to(dev) for v in (A, b, R, mx))
    tx = torch.empty(2 * n * nrhs, dtype=torch.float64, device=dev)
    tg = torch.empty(1, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream()
    pidcuda.linearsolve_verify_dev(n, nrhs, tA, n, tb, n, tR, n, tm, n, tx, n, tg, form=form,
                                   stream=s)
    s.synchronize()
    assert np.array_equal(bits(tx.cpu().numpy()), bits(x))
    assert float(tg.cpu()[0]) == G


def _pad(vec_kv_or_pt, rows, cols, ld, width):
    """Column-major (rows x cols) buffer of `width` doubles per entry -> ld-padded copy."""
    src = np.asarray(vec_kv_or_pt).reshape(cols, rows, width)
    out = np.full((cols, ld, width), np.nan)
    out[:, :rows, :] = src
    return out.reshape(-1)


@pytest.mark.parametrize("form", [pidcuda.FORM_PLAIN, pidcuda.FORM_OZAKI])
def test_ilss_device_form_padded_leading_dimensions(cuda_lib, form):
    import torch
    n, nrhs = 70, 3
    rng = np.random.default_rng(77 + form)
    A, b, R, mx = system(rng, n, nrhs, 2.0 ** -30)
    x, G = pidcuda.linearsolve_verify(A, b, R, mx, n, nrhs, form=form)
    lda, ldb, ldr, ldm, ldx = n + 3, n + 5, n + 2, n + 1, n + 4
    dev = torch.device("cuda")
    t = lambda v: torch.from_numpy(v).to(dev)
    tA, tb = t(_pad(A, n, n, lda, 2)), t(_pad(b, n, nrhs, ldb, 2))
    tR, tm = t(_pad(R, n, n, ldr, 1)), t(_pad(mx, n, nrhs, ldm, 1))
    tx = torch.full((ldx * nrhs * 2,), float("nan"), dtype=torch.float64, device=dev)
    tg = torch.empty(1, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream()
    pidcuda.linearsolve_verify_dev(n, nrhs, tA, lda, tb, ldb, tR, ldr, tm, ldm, tx, ldx, tg,
                                   form=form, stream=s)
    s.synchronize()
    got = tx.cpu().numpy().reshape(nrhs, ldx, 2)[:, :n, :].reshape(-1)
    assert np.array_equal(bits(got), bits(x))
    assert float(tg.cpu()[0]) == G


def test_ilss_nonfinite_input_reported(cuda_lib):
    from vcp_gb300.errors import NonFiniteError
    n = 40
    rng = np.random.default_rng(4)
    A, b, R, mx = system(rng, n, 1, 2.0 ** -30)
    A[2 * 17 + 1] = np.inf
    with pytest.raises(NonFiniteError):
        pidcuda.linearsolve_verify(A, b, R, mx, n, 1, form=pidcuda.FORM_OZAKI)
