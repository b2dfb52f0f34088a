"""CPU tests of the host side of pddblas's refinement consumers
(vcp_gb300.pddcuda.linearsolve / inv / cholesky, vcp/pddblas.hpp:413-563).

On the GPU their accurate products run through vcpcu_ddgemm; here the same
loops run with the oracle's bit-exact restatement of pddblas::mulmm in its
place, and must reach what the reference's own loops reached on the golden
systems (tests/golden: pddblas::linearsolve, inv, Cholesky, run by the
reference build with project-written LU / Cholesky / triangular solves).
The double-precision steps differ in their last bits (LAPACK here, the
project's LU in the reference build), so the converged dd results are
compared to 2^-96 relative, far below double precision."""
import numpy as np
import pytest

from vcp_gb300 import pddcuda


@pytest.fixture
def cpu_products(monkeypatch, oracle):
    def mulmm(A, B, m, n, k, slices=0, with_bound=True):
        return oracle.pddblas_mulmm(m, n, k, np.ascontiguousarray(A), np.ascontiguousarray(B)), None
    monkeypatch.setattr(pddcuda, "mulmm", mulmm)


def value(X):
    return X[0::2] + X[1::2]


def close(X, Y, tol=2.0 ** -96):
    scale = max(1.0, float(np.max(np.abs(value(Y)))))
    d = np.abs((X[0::2] - Y[0::2]) + (X[1::2] - Y[1::2]))
    return float(np.max(d)) <= tol * scale


def test_linearsolve_reaches_reference(cpu_products, golden):
    for idx in range(int(golden["n_pls"][0])):
        n, nrhs = (int(v) for v in golden[f"pls{idx}_shape"])
        x = pddcuda.linearsolve(golden[f"pls{idx}_A"], golden[f"pls{idx}_b"], n, nrhs)
        assert close(x, golden[f"pls{idx}_x"]), idx


def test_inv_and_cholesky_reach_reference(cpu_products, golden):
    n = int(golden["inv_n"][0])
    assert close(pddcuda.inv(golden["inv_A"], n), golden["inv_R"])
    n = int(golden["chol_n"][0])
    U = pddcuda.cholesky(golden["chol_A"], n)
    assert close(U, golden["chol_U"])
    Um = U.reshape(n, n, 2)              # Um[j, i] = entry (i, j)
    assert np.all(Um[np.triu_indices(n, 1)] == 0.0)   # every entry below the diagonal


def test_dd_add_is_kv_addition():
    from fractions import Fraction as F
    rng = np.random.default_rng(3)
    x1 = rng.standard_normal(200)
    x2 = x1 * 2.0 ** -53 * rng.uniform(-1, 1, 200)
    y1 = rng.standard_normal(200) * 2.0 ** rng.integers(-60, 60, 200)
    y2 = y1 * 2.0 ** -53 * rng.uniform(-1, 1, 200)
    s1, s2 = pddcuda.dd_add(x1, x2, y1, y2)
    for i in range(200):
        exact = F(x1[i]) + F(x2[i]) + F(y1[i]) + F(y2[i])
        got = F(s1[i]) + F(s2[i])
        assert abs(got - exact) <= abs(exact) * F(2) ** -100 + F(2) ** -1074


def eig_close(lam, X, lam_ref, X_ref, n, tol=2.0 ** -90):
    """Eigenvalues to tol relative to the largest; eigenvectors to tol per
    column after matching each column's sign to the reference's."""
    scale = float(np.max(np.abs(lam_ref[0::2])))
    dl = np.abs((lam[0::2] - lam_ref[0::2]) + (lam[1::2] - lam_ref[1::2]))
    if float(np.max(dl)) > tol * scale:
        return False
    Xh, Xl = X[0::2].reshape(n, n, order="F"), X[1::2].reshape(n, n, order="F")
    Rh, Rl = X_ref[0::2].reshape(n, n, order="F"), X_ref[1::2].reshape(n, n, order="F")
    for j in range(n):
        i = int(np.argmax(np.abs(Rh[:, j])))
        sg = 1.0 if (Xh[i, j] > 0) == (Rh[i, j] > 0) else -1.0
        d = np.abs((sg * Xh[:, j] - Rh[:, j]) + (sg * Xl[:, j] - Rl[:, j]))
        if float(np.max(d)) > tol * float(np.max(np.abs(Rh[:, j]))):
            return False
    return True


def test_eigsym_and_eigsymge_reach_reference(cpu_products, golden):
    n = int(golden["eig_n"][0])
    lam, X = pddcuda.eigsym(golden["eig_A"], n)
    assert eig_close(lam, X, golden["eig_lam"], golden["eig_X"], n)
    n = int(golden["eigge_n"][0])
    lam, X = pddcuda.eigsymge(golden["eigge_A"], golden["eigge_B"], n)
    assert eig_close(lam, X, golden["eigge_lam"], golden["eigge_X"], n)
