"""CPU tests of the Emden pipeline's host side (no GPU).

* Legendre tables: the node enclosures contain the Gauss-Legendre nodes,
  the weights sum to an interval containing 1, the basis functions match the
  reference's definition phi_i = t (1 - t) P~'_{i-1} / (i (i - 1))
  (vcp/ldbase.hpp:155-181) and the one-dimensional Gram / stiffness
  matrices OneDimL / OneDimDL of dphidphi (:1165-1186) up to rounding;
* the even list and the point counts follow the reference's index
  arithmetic (even_list_set :279-312, setting :712-753);
* the stiffness matrix DL (exact rationals, rounded outward) encloses the
  quadrature of grad phi_r . grad phi_s;
* the oracle's tensor-basis restatement encloses the exact products;
* the whole pipeline on the CPU (oracle products) verifies a solution of
  -Laplace u = u^2 at M = 10 and 20, and the H^1_0 bound shrinks with M.
"""
import numpy as np
import pytest

from vcp_gb300 import emden as E
from vcp_gb300 import legendre as L

pytest.importorskip("mpmath")


def test_tables_enclose_gauss_rule_and_basis():
    M, n = 12, 20
    T = L.basis_tables(M, n, use_cache=False)
    x, w = np.polynomial.legendre.leggauss(n)
    t = (x + 1) / 2
    assert np.all(T["x_lo"] <= T["x_hi"]) and np.all(T["w_lo"] <= T["w_hi"])
    assert np.max(np.abs(t - T["x_mid"])) < 1e-15
    assert np.max(np.abs(w / 2 - T["w_mid"])) < 1e-14
    assert T["w_lo"].sum() <= 1.0 + 1e-15 and T["w_hi"].sum() >= 1.0 - 1e-15
    from numpy.polynomial import legendre as npl
    tm = T["x_mid"]
    for a in range(M):
        i = a + 2
        c = np.zeros(i)
        c[i - 1] = 1
        ref = tm * (1 - tm) * 2 * npl.legval(2 * tm - 1, npl.legder(c)) / (i * (i - 1))
        assert np.max(np.abs(ref - T["phi_mid"][a])) < 1e-14
        dd = -2 * npl.legval(2 * tm - 1, npl.legder(c))   # phi'' = -2 P'_{i-1}(2 t - 1)
        assert np.max(np.abs(dd - T["dd_mid"][a])) < 1e-10 * max(1, np.max(np.abs(dd)))
    assert np.all(T["phi_lo"] <= T["phi_mid"]) and np.all(T["phi_mid"] <= T["phi_hi"])


def test_one_dimensional_matrices_match_quadrature():
    M, n = 10, 14
    T = L.basis_tables(M, n, use_cache=False)
    P, W = T["phi_mid"], T["w_mid"]
    Lq = (P * W) @ P.T
    L1, D1 = E._one_dim(M)
    for i in range(M):
        for j in range(M):
            assert abs(Lq[i, j] - float(L1[i][j])) < 1e-15
    # phi_{i+2}' = -P~_{i+1}: int phi' phi' = delta / (2 i + 3)
    xm = T["x_mid"]
    from numpy.polynomial import legendre as npl
    dphi = np.array([-npl.legval(2 * xm - 1, np.eye(a + 2)[a + 1]) for a in range(M)])
    Dq = (dphi * W) @ dphi.T
    for i in range(M):
        assert abs(Dq[i, i] - float(D1[i])) < 1e-15


def test_even_list_and_point_counts_follow_the_reference():
    M = 7
    ia, ib = E.even_list(M)
    # even_list_set for dim = 2, restated loop by loop
    mmax, mn = M, (M + 1) // 2
    lst = np.zeros((mn * mn, 2), dtype=int)
    ii = 0
    for d in range(2):
        lower = mn ** (2 - d - 1)
        upper = mn ** (2 - d)
        for j in range(mn ** d):
            for i in range(0, mmax, 2):
                for k in range(lower):
                    lst[ii * lower + j * upper + k, d] = i
                ii += 1
            ii = 0
    assert np.array_equal(lst[:, 0], ia) and np.array_equal(lst[:, 1], ib)
    assert E.npts_inverse(20) == 36 and E.npts_residual(20) == 46
    assert E.npts_inverse(70) == 112 and E.npts_residual(70) == 146


def test_stiffness_encloses_quadrature():
    M = 8
    ia, ib = E.even_list(M)
    lo, hi, mid = E.stiffness(M, ia, ib)
    assert np.all(lo <= mid) and np.all(mid <= hi)
    T = L.basis_tables(M, 12, use_cache=False)
    from numpy.polynomial import legendre as npl
    xm, W = T["x_mid"], T["w_mid"]
    ph = T["phi_mid"]
    dph = np.array([-npl.legval(2 * xm - 1, np.eye(a + 2)[a + 1]) for a in range(M)])
    n = ia.size
    DLq = np.zeros((n, n))
    for r in range(n):
        for s in range(n):
            gx = np.sum(W * dph[ia[r]] * dph[ia[s]]) * np.sum(W * ph[ib[r]] * ph[ib[s]])
            gy = np.sum(W * ph[ia[r]] * ph[ia[s]]) * np.sum(W * dph[ib[r]] * dph[ib[s]])
            DLq[r, s] = gx + gy
    assert np.max(np.abs(DLq - mid)) < 1e-15


def test_oracle_tensor_basis_encloses_products():
    from oracle import oracle as O
    rng = np.random.default_rng(4)
    nt, nqa, nqb = 5, 4, 3
    P = nqa * nqb
    base = rng.standard_normal((nt, nqa))
    Ta = E.table_kv(base - 1e-12, base + 1e-12)
    baseb = rng.standard_normal((nt, nqb))
    Tb = E.table_kv(baseb - 1e-12, baseb + 1e-12)
    s = rng.standard_normal(P)
    s1 = E.table_kv(s[None, :] - 1e-9, s[None, :] + 1e-9)
    ia = np.array([0, 4, 2], dtype=np.int32)
    ib = np.array([1, 1, 0], dtype=np.int32)
    out = np.zeros(2 * 3 * P)
    O.tensor_basis(3, ia, ib, nt, Ta, Tb, nqa, nqb, out, 3, s1=s1)
    for i in range(3):
        for q in range(P):
            qa, qb = divmod(q, nqb)
            v = base[ia[i], qa] * baseb[ib[i], qb] * s[q]
            lo, hi = out[2 * (i + q * 3)], out[2 * (i + q * 3) + 1]
            assert lo <= v <= hi and hi - lo < 1e-8 * max(1, abs(v))
    outT = np.zeros(2 * 3 * P)
    O.tensor_basis(3, ia, ib, nt, Ta, Tb, nqa, nqb, outT, P, s1=s1, transposed=True)
    assert np.array_equal(outT.reshape(3, P, 2).transpose(1, 0, 2).ravel(), out)


def test_cpu_pipeline_verifies_emden():
    from oracle.emden_host import HostProducts
    r10 = E.verify(10, HostProducts())
    r20 = E.verify(20, HostProducts())
    for r in (r10, r20):
        assert r.verified and r.kantorovich <= 0.5
        assert 29.0 < r.uh_max < 31.0
        assert 1.0 <= r.K < 10.0
    assert r20.error_bound_H10 < r10.error_bound_H10 < 10.0
    assert r20.error_bound_H10 < 1e-3
