"""GPU parity of the device-resident verification of imats::eigsymge
(vcp/imats.hpp:419-522: vcpcu_ieigsymge and its two stages).

* Plain form: every bit of the merged enclosures equals the reference's own
  eigsymge (golden vectors, made with its X, lambda and Y) and the
  restatement (pinned to the reference) on random problems; the midpoints
  handed to the caller's inverse are the restatement's.
* Tensor-core form: bit-identical to the restatement fed with the GPU's own
  products ([A]X, [B]X, YC, Y[BX] -- each bit-identical to the host model
  elsewhere).
"""
import ctypes
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


def problem(rng, n, rel, spread=0.1):
    Am = rng.standard_normal((n, n))
    Am = (Am + Am.T) / 2
    Bm = np.eye(n) + spread * rng.standard_normal((n, n))
    Bm = Bm @ Bm.T
    A = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * rel)
    B = W._kv(Bm.ravel(order="F"), np.abs(Bm.ravel(order="F")) * rel)
    return A, B, Am, Bm


def eigenpairs(Am, Bm):
    """Approximate eigenpairs of Am x = l Bm x (B-orthonormal X), any method."""
    L = np.linalg.cholesky(Bm)
    Li = np.linalg.inv(L)
    w, V = np.linalg.eigh(Li @ Am @ Li.T)
    X = Li.T @ V
    return X.ravel(order="F").copy(), w.copy()


def test_eigsymge_plain_matches_reference_golden(cuda_lib, oracle):
    g = np.load(GOLDEN)
    for idx in range(int(g["n_ge"][0])):
        n = int(g[f"ge{idx}_n"][0])
        A, B, X = g[f"ge{idx}_A"], g[f"ge{idx}_B"], g[f"ge{idx}_X"]
        seen = {}

        def inverse(M, Y=g[f"ge{idx}_Y"], n=n):
            seen["M"] = M.ravel(order="F").copy()
            return Y.reshape(n, n, order="F")

        lam, bound = pidcuda.eigsymge_verify(A, B, X, g[f"ge{idx}_lambda"], n, inverse,
                                             form=pidcuda.FORM_PLAIN)
        assert bound == float(g[f"ge{idx}_bound"][0]), idx
        assert np.array_equal(bits(lam), bits(g[f"ge{idx}_lam"])), idx
        BX = oracle.pidblas_mul_point(0, n, n, n, B, X)
        mid, _ = oracle.midrad(BX)
        assert np.array_equal(bits(seen["M"]), bits(mid)), idx


@pytest.mark.parametrize("n", [2, 10, 64, 130])
def test_eigsymge_plain_matches_restatement(cuda_lib, oracle, n):
    rng = np.random.default_rng(n)
    A, B, Am, Bm = problem(rng, n, 2.0 ** -30)
    X, lmb = eigenpairs(Am, Bm)
    used = {}

    def inverse(M):
        used["Y"] = np.linalg.inv(M)
        return used["Y"]

    lam, bound = pidcuda.eigsymge_verify(A, B, X, lmb, n, inverse, form=pidcuda.FORM_PLAIN)
    Y = used["Y"].ravel(order="F").copy()
    st, lo, bo = oracle.ieigsymge(n, A, B, X, lmb, Y)
    assert st == 0 and bound == bo
    assert np.array_equal(bits(lam), bits(lo))


def test_eigsymge_imats_loop_kernel_bitexact(cuda_lib, oracle):
    """The base-class kv loop product R = Y C on its own (through stage 2's
    plain path) against its restatement, with signed zeros and mixed signs."""
    import torch
    n = 70
    rng = np.random.default_rng(5)
    A, B, Am, Bm = problem(rng, n, 2.0 ** -30)
    X, lmb = eigenpairs(Am, Bm)
    Xr = X.copy()
    Xr[[5, 400, 1234]] = 0.0  # a few signed zeros, X stays well conditioned
    Xr[[17, 999]] = -0.0
    dev = torch.device("cuda")
    s = torch.cuda.current_stream()
    tA, tB, tX, tl = (torch.from_numpy(v).to(dev) for v in (A, B, Xr, lmb))
    C = torch.empty(2 * n * n, dtype=torch.float64, device=dev)
    BX = torch.empty_like(C)
    M = torch.empty(n * n, dtype=torch.float64, device=dev)
    pidcuda.eigsymge_stage1_dev(n, tA, n, tB, n, tX, n, C, BX, M, pidcuda.FORM_PLAIN, 0, s)
    Y = np.linalg.inv(M.cpu().numpy().reshape(n, n, order="F")).ravel(order="F").copy()
    Yd = torch.from_numpy(Y).to(dev)
    lam = torch.empty(2 * n, dtype=torch.float64, device=dev)
    bound = torch.empty(1, dtype=torch.float64, device=dev)
    pidcuda.eigsymge_stage2_dev(n, tl, Yd, n, C, BX, lam, bound, pidcuda.FORM_PLAIN, 0, s)
    s.synchronize()
    st, lo, bo = oracle.ieigsymge(n, A, B, Xr, lmb, Y, merge=False)
    assert st == 0 and float(bound.cpu()[0]) == bo
    assert np.array_equal(bits(lam.cpu().numpy()), bits(lo))
    Cp = C.cpu().numpy()  # C - BX Lambda after stage 2
    R = oracle.imats_mul_m_im_naive(n, n, n, Y, Cp)
    assert np.all(np.isfinite(R))


@pytest.mark.parametrize("n", [64, 200])
def test_eigsymge_ozaki_matches_restatement(cuda_lib, oracle, n):
    import torch
    rng = np.random.default_rng(100 + n)
    A, B, Am, Bm = problem(rng, n, 2.0 ** -36)
    X, lmb = eigenpairs(Am, Bm)
    dev = torch.device("cuda")
    s = torch.cuda.current_stream()
    tA, tB, tX, tl = (torch.from_numpy(v).to(dev) for v in (A, B, X, lmb))
    C = torch.empty(2 * n * n, dtype=torch.float64, device=dev)
    BX = torch.empty_like(C)
    M = torch.empty(n * n, dtype=torch.float64, device=dev)
    f = pidcuda.FORM_OZAKI
    pidcuda.eigsymge_stage1_dev(n, tA, n, tB, n, tX, n, C, BX, M, f, 0, s)
    C_in, BX_in = C.cpu().numpy(), BX.cpu().numpy()
    Y = np.linalg.inv(M.cpu().numpy().reshape(n, n, order="F")).ravel(order="F").copy()
    lam = torch.empty(2 * n, dtype=torch.float64, device=dev)
    bound = torch.empty(1, dtype=torch.float64, device=dev)
    pidcuda.eigsymge_stage2_dev(n, tl, torch.from_numpy(Y).to(dev), n, C, BX, lam, bound, f, 0, s)
    s.synchronize()
    Cp = C.cpu().numpy()
    R_in = pidcuda.mul_point(1, Y, Cp, n, n, n, form=f)
    S_in = pidcuda.mul_point(1, Y, BX_in, n, n, n, form=f)
    st, lo, bo = oracle.ieigsymge(n, A, B, X, lmb, Y, C=C_in, BX=BX_in, R=R_in, S=S_in,
                                  merge=False)
    assert st == 0 and float(bound.cpu()[0]) == bo
    assert np.array_equal(bits(lam.cpu().numpy()), bits(lo))
    # the enclosures hold the eigenvalues of the midpoint problem
    mid = lam.cpu().numpy()
    assert np.all(mid[0::2] <= lmb + 1e-9 * np.abs(lmb).max())
    assert np.all(mid[1::2] >= lmb - 1e-9 * np.abs(lmb).max())


def test_eig_merge_matches_restatement(cuda_lib, oracle):
    rng = np.random.default_rng(9)
    c = np.sort(rng.uniform(0, 10, 60))
    w = rng.uniform(0, 0.4, 60)
    lam = np.empty(120)
    lam[0::2], lam[1::2] = c - w, c + w
    ours = pidcuda.eig_merge(lam.copy(), 60)
    ref = lam.copy()
    oracle.lib().orc_eig_merge(60, oracle._p(ref))
    assert np.array_equal(bits(ours), bits(ref))


def test_eigsymge_failed_check_raises(cuda_lib):
    n = 8
    rng = np.random.default_rng(2)
    A, B, Am, Bm = problem(rng, n, 0.5)
    X, lmb = eigenpairs(Am, Bm)
    _, bound = pidcuda.eigsymge_verify(A, B, X, lmb, n, form=pidcuda.FORM_PLAIN, check=False)
    assert bound >= 1.0
    with pytest.raises(VerificationError):
        pidcuda.eigsymge_verify(A, B, X, lmb, n, form=pidcuda.FORM_PLAIN)


def test_eigsymge_stages_padded_leading_dimensions(cuda_lib):
    import torch
    n = 50
    rng = np.random.default_rng(31)
    A, B, Am, Bm = problem(rng, n, 2.0 ** -30)
    X, lmb = eigenpairs(Am, Bm)
    used = {}

    def inverse(M):
        used["Y"] = np.linalg.inv(M)
        return used["Y"]

    lam_ref, bound_ref = pidcuda.eigsymge_verify(A, B, X, lmb, n, inverse,
                                                 form=pidcuda.FORM_PLAIN)
    Y = used["Y"].ravel(order="F").copy()

    def pad(v, ld, width):
        out = np.full((n, ld, width), np.nan)
        out[:, :n, :] = np.asarray(v).reshape(n, n, width)
        return out.reshape(-1)

    lda, ldb, ldx, ldy = n + 2, n + 7, n + 1, n + 3
    dev = torch.device("cuda")
    t = lambda v: torch.from_numpy(v).to(dev)
    tA, tB, tX, tY, tl = t(pad(A, lda, 2)), t(pad(B, ldb, 2)), t(pad(X, ldx, 1)), \
        t(pad(Y, ldy, 1)), t(lmb)
    C = torch.empty(2 * n * n, dtype=torch.float64, device=dev)
    BX = torch.empty_like(C)
    M = torch.empty(n * n, dtype=torch.float64, device=dev)
    lam = torch.empty(2 * n, dtype=torch.float64, device=dev)
    bound = torch.empty(1, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream()
    pidcuda.eigsymge_stage1_dev(n, tA, lda, tB, ldb, tX, ldx, C, BX, M, pidcuda.FORM_PLAIN, 0, s)
    pidcuda.eigsymge_stage2_dev(n, tl, tY, ldy, C, BX, lam, bound, pidcuda.FORM_PLAIN, 0, s)
    s.synchronize()
    merged = pidcuda.eig_merge(lam.cpu().numpy().copy(), n)
    assert np.array_equal(bits(merged), bits(lam_ref))
    assert float(bound.cpu()[0]) == bound_ref
