"""GPU parity of the dd GEMM (pddblas::mulmm semantics, vcpcu_ddgemm):
bit-identical to the exact-integer host model (tests/dd_model.py), and the
returned bound holds against the exact product (Python rationals)."""
from fractions import Fraction

import numpy as np
import pytest

from vcp_gb300 import pddcuda
from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dd_matrix(rng, rows, cols, phi):
    hi = W.ephi(rng, rows * cols, phi)
    lo = hi * 2.0 ** -53 * rng.uniform(-1, 1, rows * cols)
    out = np.empty(2 * rows * cols)
    out[0::2], out[1::2] = hi, lo
    return out


@pytest.mark.parametrize("case", [(1, 1, 1, 13), (5, 7, 9, 13), (40, 33, 300, 13),
                                  (17, 20, 1100, 10), (30, 9, 64, 7)])
def test_ddgemm_bitexact_and_bound(cuda_lib, case):
    from tests.dd_model import ddgemm
    m, n, k, s = case
    rng = np.random.default_rng(m + 10 * n + k)
    A = dd_matrix(rng, m, k, 16)
    B = dd_matrix(rng, k, n, 16)
    C, E = pddcuda.mulmm(A, B, m, n, k, slices=s)
    Cm, Em = ddgemm(m, n, k, list(A), list(B), slices=s)
    assert np.array_equal(C.view(np.int64), np.array(Cm).view(np.int64))
    assert np.array_equal(E.view(np.int64), np.array(Em).view(np.int64))
    for t in range(0, m * n, max(1, (m * n) // 50)):
        i, j = t % m, t // m
        exact = sum((Fraction(A[2 * (i + p * m)]) + Fraction(A[2 * (i + p * m) + 1])) *
                    (Fraction(B[2 * (p + j * k)]) + Fraction(B[2 * (p + j * k) + 1]))
                    for p in range(k))
        assert abs(exact - Fraction(C[2 * t]) - Fraction(C[2 * t + 1])) <= Fraction(E[t])


def test_ddgemm_accuracy_vs_exact(cuda_lib, oracle):
    """Relative error of the dd midpoint against the exact product (long
    accumulator over the four double products of each dd pair)."""
    rng = np.random.default_rng(5)
    m = n = 64
    k = 1024
    A = dd_matrix(rng, m, k, 0)
    B = dd_matrix(rng, k, n, 0)
    C, E = pddcuda.mulmm(A, B, m, n, k)
    # expand dd pairs: A2 (m x 2k) = [hi | lo], B2 (2k x n) = [hi ; lo] twice
    Ahi, Alo = A[0::2].reshape(k, m).T, A[1::2].reshape(k, m).T
    Bhi, Blo = B[0::2].reshape(n, k).T, B[1::2].reshape(n, k).T
    A4 = np.hstack([Ahi, Ahi, Alo, Alo]).ravel(order="F")
    B4 = np.vstack([Bhi, Blo, Bhi, Blo]).ravel(order="F")
    rows = np.repeat(np.arange(m), n)
    cols = np.tile(np.arange(n), m)
    dn, up = oracle.exact_dot(m, n, 4 * k, A4, B4, rows, cols)
    idx = rows + cols * m
    c = C[0::2][idx] + C[1::2][idx]
    # the exact value lies in [dn, up] (adjacent doubles); the dd is far more accurate
    assert np.all(np.abs(C[0::2][idx] - dn) <= np.abs(dn) * 2.0 ** -50)
    assert np.all(E[idx] <= np.maximum(np.abs(dn), 1.0) * 2.0 ** -80)


@pytest.mark.parametrize("phi", [0, 16])
def test_ddgemm_accuracy_against_pddblas(cuda_lib, oracle, phi):
    """Against the exact product (long accumulator), next to pddblas::mulmm
    (the reference's Ozaki scheme, vcp/pddblas.hpp:318-376, restated bit
    for bit by the oracle): the GPU's median relative error is no larger
    than pddblas's; its largest stays below 2^-96 (the 112-bit operands are
    truncated relative to the row / column maxima, so entries much smaller
    than those products keep fewer bits -- up to about 50x pddblas's
    largest error at phi = 16, where pddblas keeps ~150 bits per slice
    stack); and the returned bound holds on every entry."""
    rng = np.random.default_rng(40 + phi)
    m, n, k = 48, 40, 2100
    A = dd_matrix(rng, m, k, phi)
    B = dd_matrix(rng, k, n, phi)
    C, E = pddcuda.mulmm(A, B, m, n, k)
    P = oracle.pddblas_mulmm(m, n, k, A, B)
    rows = np.repeat(np.arange(m), n).astype(np.int32)
    cols = np.tile(np.arange(n), m).astype(np.int32)
    eg, ab = oracle.dd_residual(m, n, k, A, B, C, rows, cols)
    ep, _ = oracle.dd_residual(m, n, k, A, B, P, rows, cols)
    scale = np.where(ab > 0, ab, 1.0)
    assert np.median(eg / scale) <= np.median(ep / scale)
    assert np.max(eg / scale) <= 2.0 ** -96
    assert np.all(eg <= E[rows + cols * m])


def test_dd_mulltmm_on_gpu(cuda_lib, oracle):
    """pddblas::mulltmm (A^T A, vcp/pddblas.hpp:379-409) on the GPU: the dd
    product of A^T and A with the lower triangle taken from the upper one,
    as the reference does; exactly symmetric, bound holding against the
    exact A^T A, median error no larger than the reference's own."""
    rng = np.random.default_rng(77)
    k, n = 700, 33
    A = dd_matrix(rng, k, n, 8)
    C, E = pddcuda.mulltmm(A, n, k)
    Cm = C.reshape(n, n, 2)
    assert np.array_equal(Cm.view(np.int64), Cm.transpose(1, 0, 2).view(np.int64))
    At = A.reshape(n, k, 2).transpose(1, 0, 2).copy().reshape(-1)
    rows = np.repeat(np.arange(n), n).astype(np.int32)
    cols = np.tile(np.arange(n), n).astype(np.int32)
    eg, ab = oracle.dd_residual(n, n, k, At, A, C, rows, cols)
    assert np.all(eg <= E[rows + cols * n])
    P = oracle.pddblas_mulltmm(k, n, A)
    ep, _ = oracle.dd_residual(n, n, k, At, A, P, rows, cols)
    scale = np.where(ab > 0, ab, 1.0)
    assert np.median(eg / scale) <= np.median(ep / scale)
    assert np.max(eg / scale) <= 2.0 ** -96


def _close(X, Y, tol=2.0 ** -96):
    scale = max(1.0, float(np.max(np.abs(Y[0::2]))))
    return float(np.max(np.abs((X[0::2] - Y[0::2]) + (X[1::2] - Y[1::2])))) <= tol * scale


def test_pddblas_refinements_on_gpu_reach_reference(cuda_lib, golden):
    """pddblas::linearsolve / inv / Cholesky (vcp/pddblas.hpp:413-563) with
    their accurate products on the GPU reach the reference's own results on
    the golden systems (to 2^-96 relative: the double-precision steps differ
    in last bits between LAPACK and the reference build's solves)."""
    for idx in range(int(golden["n_pls"][0])):
        n, nrhs = (int(v) for v in golden[f"pls{idx}_shape"])
        x = pddcuda.linearsolve(golden[f"pls{idx}_A"], golden[f"pls{idx}_b"], n, nrhs)
        assert _close(x, golden[f"pls{idx}_x"]), idx
    n = int(golden["inv_n"][0])
    assert _close(pddcuda.inv(golden["inv_A"], n), golden["inv_R"])
    n = int(golden["chol_n"][0])
    assert _close(pddcuda.cholesky(golden["chol_A"], n), golden["chol_U"])


def test_pddblas_linearsolve_on_gpu_residual(cuda_lib, oracle):
    """A 600 x 600 dd system solved with the GPU products: the exact residual
    |A x - b| (long accumulator) is at dd level."""
    rng = np.random.default_rng(9)
    n, nrhs = 600, 2
    A = dd_matrix(rng, n, n, 2)
    A[0::2][np.arange(n) * (n + 1)] += 4.0 * n
    b = dd_matrix(rng, n, nrhs, 2)
    x = pddcuda.linearsolve(A, b, n, nrhs)
    rows = np.repeat(np.arange(n), nrhs).astype(np.int32)
    cols = np.tile(np.arange(nrhs), n).astype(np.int32)
    err, ab = oracle.dd_residual(n, nrhs, n, A, x, b, rows, cols)
    assert np.max(err) <= 2.0 ** -95 * np.max(ab)


def test_pddblas_eigen_refinements_on_gpu_reach_reference(cuda_lib, golden):
    """pddblas::eigsym / eigsymge (Ogita-Aishima refinement,
    vcp/pddblas.hpp:221-314, 566-657) with every product on the GPU: the
    eigenvalues and (sign-matched) eigenvectors reach the reference's own to
    2^-90 relative."""
    from tests.test_pddcuda_host import eig_close
    n = int(golden["eig_n"][0])
    lam, X = pddcuda.eigsym(golden["eig_A"], n)
    assert eig_close(lam, X, golden["eig_lam"], golden["eig_X"], n)
    n = int(golden["eigge_n"][0])
    lam, X = pddcuda.eigsymge(golden["eigge_A"], golden["eigge_B"], n)
    assert eig_close(lam, X, golden["eigge_lam"], golden["eigge_X"], n)
