"""CPU tests: the oracle pinned against the reference.

* golden vectors produced by the reference's own code (tests/golden/golden.npz,
  made by tests/golden/make_golden.py from vblas rmatmul and
  vcp::matrix<interval, pidblas>);
* where the reference sources are mounted, live bit-for-bit comparison with
  the reference compiled from its tree (oracle/_ref);
* the known-answer rounding tests of vblas/Check_rmatmul_rounding.cpp:51-116
  and vblas/Check_udmatmul_rounding.cpp:40-102 (every entry must differ
  between the upward and downward products);
* self-tests of the exact accumulator against Python's exact rationals.
"""
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from vcp_gb300 import workloads as W

def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def test_oracle_rmatmul_matches_golden(oracle, golden):
    for idx in range(int(golden["n_rm"][0])):
        m, n, k = map(int, golden[f"rm{idx}_shape"])
        A, B = golden[f"rm{idx}_A"], golden[f"rm{idx}_B"]
        for rnd, tag in ((1, "up"), (-1, "dn"), (0, "rn")):
            got = oracle.rmatmul(m, n, k, A, B, rnd)
            assert np.array_equal(bits(got), bits(golden[f"rm{idx}_{tag}"])), (idx, tag)


def test_oracle_pidblas_matches_golden(oracle, golden):
    for idx in range(int(golden["n_iv"][0])):
        m, n, k = map(int, golden[f"iv{idx}_shape"])
        got = oracle.pidblas_mulmm(m, n, k, golden[f"iv{idx}_A"], golden[f"iv{idx}_B"])
        assert np.array_equal(bits(got), bits(golden[f"iv{idx}_C"])), idx


@pytest.mark.parametrize("shape", [(1, 1, 1), (31, 257, 17), (100, 513, 12), (16, 1000, 5)])
def test_oracle_rmatmul_matches_reference_build(oracle, shape):
    if oracle.ref_lib() is None:
        from oracle.build import build_reference
        if build_reference() is None:
            pytest.skip("reference sources not mounted")
    m, n, k = shape
    rng = np.random.default_rng(sum(shape))
    A, B = W.ephi(rng, m * n, 32), W.ephi(rng, n * k, 32)
    for rnd in (1, -1, 0):
        assert np.array_equal(bits(oracle.rmatmul(m, n, k, A, B, rnd)),
                              bits(oracle.ref_rmatmul(m, n, k, A, B, rnd)))


def test_oracle_pidblas_matches_reference_build(oracle):
    if oracle.ref_lib() is None:
        from oracle.build import build_reference
        if build_reference() is None:
            pytest.skip("reference sources not mounted")
    rng = np.random.default_rng(5)
    for m, n, k in [(48, 40, 100), (1, 30, 20), (30, 1, 20), (25, 25, 1)]:
        A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
        B = W.interval_ephi(rng, k, n, 4, 2.0 ** -10)
        assert np.array_equal(bits(oracle.pidblas_mulmm(m, n, k, A, B)),
                              bits(oracle.ref_pidblas_mulmm(m, n, k, A, B)))


def kat_patterns(n):
    """The two patterns of vblas/Check_rmatmul_rounding.cpp (column-major A, B)."""
    pats = []
    for i in (0, n // 2, n - 1):  # 1/3 rank-1 pattern (:55-79), a few i
        A = np.zeros((n, n)); B = np.zeros((n, n))
        A[:, i] = 1.0 / 3.0; B[i, :] = 1.0 / 3.0
        pats.append((A.ravel(order="F"), B.ravel(order="F")))
    for i in (2, n // 2, n - 1):  # 1 + 2^-54 pattern (:83-114)
        A = np.zeros((n, n)); B = np.zeros((n, n))
        A[:, 1] = 1.0; B[1, :] = 1.0
        A[:, i] = 2.0 ** -27; B[i, :] = 2.0 ** -27
        pats.append((A.ravel(order="F"), B.ravel(order="F")))
    return pats


def test_oracle_rounding_kat(oracle):
    n = 90
    for A, B in kat_patterns(n):
        cu = oracle.rmatmul(n, n, n, A, B, 1)
        cd = oracle.rmatmul(n, n, n, A, B, -1)
        assert np.all(cu > cd)


def test_exact_sum_matches_fractions(oracle):
    rng = np.random.default_rng(3)
    for trial in range(20):
        x = rng.standard_normal(200) * np.exp2(rng.integers(-300, 300, 200))
        if trial % 4 == 0:
            x[:5] = [5e-324, -5e-324, 1e308, -1e308, 2.0 ** -1074 * 3]
        F = sum(Fraction(float(v)) for v in x)
        lo, hi = oracle.exact_sum(x, -1), oracle.exact_sum(x, 1)
        assert Fraction(lo) <= F <= Fraction(hi)
        assert hi == lo if Fraction(lo) == F else np.nextafter(lo, np.inf) == hi


def test_exact_dot_and_hull(oracle):
    rng = np.random.default_rng(4)
    m, n, k = 6, 5, 40
    A = W.ephi(rng, m * k, 30)
    B = W.ephi(rng, k * n, 30)
    rows = np.repeat(np.arange(m), n)
    cols = np.tile(np.arange(n), m)
    dn, up = oracle.exact_dot(m, n, k, A, B, rows, cols)
    for t, (i, j) in enumerate(zip(rows, cols)):
        F = sum(Fraction(float(A[i + p * m])) * Fraction(float(B[p + j * k])) for p in range(k))
        assert Fraction(dn[t]) <= F <= Fraction(up[t])
    # interval hull: endpoints straddling zero exercise every min/max case
    Ai = W.interval_ephi(rng, m, k, 3, 0.7)
    Bi = W.interval_ephi(rng, k, n, 3, 1.3)
    lo, hi = oracle.exact_hull(m, n, k, Ai, Bi, rows, cols)
    for t, (i, j) in enumerate(zip(rows, cols)):
        L = Fraction(0); U = Fraction(0)
        for p in range(k):
            a = [Fraction(float(Ai[2 * (i + p * m) + s])) for s in (0, 1)]
            b = [Fraction(float(Bi[2 * (p + j * k) + s])) for s in (0, 1)]
            prods = [x * y for x in a for y in b]
            L += min(prods); U += max(prods)
        assert Fraction(lo[t]) <= L and U <= Fraction(hi[t])
        assert Fraction(float(np.nextafter(lo[t], np.inf))) > L  # tight: RD of the exact sum
        assert Fraction(float(np.nextafter(hi[t], -np.inf))) < U


def test_midrad_encloses(oracle):
    rng = np.random.default_rng(6)
    X = W.interval_ephi(rng, 50, 50, 40, 0.3)
    X[:4] = [-1e308, 1.7e308, 1.7e308, 1.79e308]  # lo + up overflow path
    m, r = oracle.midrad(X)
    for t in range(X.size // 2):
        lo, up = Fraction(float(X[2 * t])), Fraction(float(X[2 * t + 1]))
        assert Fraction(float(m[t])) - Fraction(float(r[t])) <= lo
        assert up <= Fraction(float(m[t])) + Fraction(float(r[t]))


def test_oracle_other_products_match_golden(oracle, golden):
    """pidblas::mul_im_m / mul_m_im / mulltmm / vmulmm and the imats::linearsolve
    bound, against vectors the reference produced."""
    for idx in range(int(golden["n_mp"][0])):
        side, m, n, k = map(int, golden[f"mp{idx}_shape"])
        got = oracle.pidblas_mul_point(side, m, n, k, golden[f"mp{idx}_L"], golden[f"mp{idx}_R"])
        assert np.array_equal(bits(got), bits(golden[f"mp{idx}_C"])), idx
    for idx in range(int(golden["n_sy"][0])):
        n, k = map(int, golden[f"sy{idx}_shape"])
        assert np.array_equal(bits(oracle.pidblas_mulltmm(n, k, golden[f"sy{idx}_A"])),
                              bits(golden[f"sy{idx}_C"])), idx
        assert np.array_equal(bits(oracle.pidblas_vmulmm(n, k, golden[f"sy{idx}_P"])),
                              bits(golden[f"sy{idx}_V"])), idx
    for idx in range(int(golden["n_nm"][0])):
        n = int(golden[f"nm{idx}_n"][0])
        g = oracle.norm_I_minus_RA(n, golden[f"nm{idx}_R"], golden[f"nm{idx}_A"])
        assert g == float(golden[f"nm{idx}_bound"][0])


def test_oracle_other_products_match_reference_build(oracle):
    import ctypes
    if oracle.ref_lib() is None:
        from oracle.build import build_reference
        if build_reference() is None:
            pytest.skip("reference sources not mounted")
    rng = np.random.default_rng(8)
    for side, m, n, k in [(0, 40, 17, 90), (1, 17, 40, 90), (0, 1, 5, 7), (1, 5, 1, 7)]:
        L = W.interval_ephi(rng, m, k, 6, 0.01) if side == 0 else W.ephi(rng, m * k, 6)
        R = W.ephi(rng, k * n, 6) if side == 0 else W.interval_ephi(rng, k, n, 6, 0.01)
        ref = np.zeros(2 * m * n)
        assert oracle.ref_call("ref_pidblas_mul_point", side, m, n, k, oracle._p(L), oracle._p(R),
                               oracle._p(ref)) == 0
        assert np.array_equal(bits(oracle.pidblas_mul_point(side, m, n, k, L, R)), bits(ref))
    n, k = 30, 70
    A = W.interval_ephi(rng, k, n, 5, 0.001)
    ref = np.zeros(2 * n * n)
    assert oracle.ref_call("ref_pidblas_mulltmm", n, k, oracle._p(A), oracle._p(ref)) == 0
    assert np.array_equal(bits(oracle.pidblas_mulltmm(n, k, A)), bits(ref))
    nn = 25
    Am = np.eye(nn) + 0.1 * rng.standard_normal((nn, nn))
    Ai = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * 1e-6)
    Rinv = np.linalg.inv(Am).ravel(order="F")
    g = ctypes.c_double(0.0)
    assert oracle.ref_call("ref_norm_I_minus_RA", nn, oracle._p(Rinv), oracle._p(Ai),
                           ctypes.addressof(g)) == 0
    assert oracle.norm_I_minus_RA(nn, Rinv, Ai) == g.value


def test_dd_residual_known_answers(oracle):
    """orc_dd_residual: exact |S - C| for a dd product with a known value."""
    import numpy as np
    A = np.array([1.0, 2.0 ** -60])          # 1 + 2^-60
    B = np.array([3.0, 0.0])
    rows = np.array([0])
    cols = np.array([0])
    err, ab = oracle.dd_residual(1, 1, 1, A, B, np.array([3.0, 3 * 2.0 ** -60]), rows, cols)
    assert err[0] == 0.0 and ab[0] == 3.0
    err, _ = oracle.dd_residual(1, 1, 1, A, B, np.array([3.0, 0.0]), rows, cols)
    assert err[0] == 3 * 2.0 ** -60
    # two terms whose hi parts cancel: S = 2^-70 exactly
    A2 = np.array([1.0, 0.0, 1.0, 2.0 ** -70])
    B2 = np.array([1.0, 0.0, -1.0, 0.0])
    err, ab = oracle.dd_residual(1, 1, 2, A2, B2, np.array([0.0, 0.0]), rows, cols)
    assert ab[0] == 2.0 ** -70 and err[0] == 2.0 ** -70


def test_ifma_oracle_golden(oracle):
    """The C restatement of vcp::ifma and pidblas_fma::mulmm reproduces the
    reference's outputs (golden vectors made by the reference build)."""
    import numpy as np
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "golden.npz")
    R = oracle.ifma(g["if_A"], g["if_B"], g["if_C"])
    assert np.array_equal(R.view(np.int64), g["if_R"].view(np.int64))
    for idx in range(int(g["n_fm"][0])):
        m, n, k = map(int, g[f"fm{idx}_shape"])
        C = oracle.pidblas_fma_mulmm(m, n, k, g[f"fm{idx}_A"], g[f"fm{idx}_B"])
        assert np.array_equal(C.view(np.int64), g[f"fm{idx}_C"].view(np.int64)), idx


def test_ifma_oracle_vs_reference_build(oracle):
    """Fresh random cases against the reference compiled here (skipped where
    the reference sources are not mounted)."""
    import numpy as np
    import pytest
    R = oracle.ref_lib()
    if R is None:
        pytest.skip("reference build unavailable")
    from tests.golden.make_golden import mixed_intervals
    rng = np.random.default_rng(99)
    n = 10000
    A, B, C = (mixed_intervals(rng, n) for _ in range(3))
    out = np.empty(2 * n)
    R.ref_ifma(n, oracle._p(A), oracle._p(B), oracle._p(C), oracle._p(out))
    assert np.array_equal(oracle.ifma(A, B, C).view(np.int64), out.view(np.int64))
    m, nn, k = 23, 19, 77
    A, B = mixed_intervals(rng, m * k), mixed_intervals(rng, k * nn)
    ref = np.empty(2 * m * nn)
    assert R.ref_pidblas_fma_mulmm(m, nn, k, oracle._p(A), oracle._p(B), oracle._p(ref)) == 0
    assert np.array_equal(oracle.pidblas_fma_mulmm(m, nn, k, A, B).view(np.int64),
                          ref.view(np.int64))


def _lss_case(rng, n, nrhs, rel, shift=4.0):
    Am = rng.uniform(-1.0, 1.0, (n, n)) + shift * np.eye(n)
    A = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * rel)
    bm = rng.uniform(-1.0, 1.0, n * nrhs)
    return A, W._kv(bm, np.abs(bm) * 2.0 ** -35)


def test_oracle_linearsolve_matches_golden(oracle, golden):
    """imats::linearsolve's verification (restated) on the reference's own
    R, mx: every bit of x, the bound, and the failing check."""
    for idx in range(int(golden["n_ls"][0])):
        n, nrhs = map(int, golden[f"ls{idx}_shape"])
        st, x, G = oracle.ilss_verify(n, nrhs, golden[f"ls{idx}_A"], golden[f"ls{idx}_b"],
                                      golden[f"ls{idx}_R"], golden[f"ls{idx}_mx"])
        assert st == int(golden[f"ls{idx}_status"][0]), idx
        assert G == float(golden[f"ls{idx}_bound"][0]), idx
        if st == 0:
            assert np.array_equal(bits(x), bits(golden[f"ls{idx}_x"])), idx


def test_oracle_linearsolve_matches_reference_build(oracle):
    """Live: the reference's imats<double, pidblas>::linearsolve (LU shim for
    its LAPACK inverse) against the restatement on the R, mx it used."""
    if oracle.ref_lib() is None:
        from oracle.build import build_reference
        if build_reference() is None:
            pytest.skip("reference sources not mounted")
    rng = np.random.default_rng(31)
    for n, nrhs, rel in [(2, 1, 2.0 ** -30), (3, 2, 2.0 ** -30), (17, 3, 2.0 ** -20),
                         (40, 1, 2.0 ** -44), (65, 6, 2.0 ** -30), (9, 1, 0.4)]:
        A, b = _lss_case(rng, n, nrhs, rel, 2.0 if rel > 0.1 else 4.0)
        st, xr, R, mx = oracle.ref_imats_linearsolve(n, nrhs, A, b)
        st2, xo, G = oracle.ilss_verify(n, nrhs, A, b, R, mx)
        assert st == st2, (n, nrhs)
        if st == 0:
            assert np.array_equal(bits(xo), bits(xr)), (n, nrhs)
    # an exact point system: the enclosure holds the rational solution
    n = 6
    M = np.round(rng.uniform(-5, 5, (n, n))) + 20 * np.eye(n)
    bb = np.round(rng.uniform(-5, 5, n))
    A = W._kv(M.ravel(order="F"), np.zeros(n * n))
    b = W._kv(bb, np.zeros(n))
    st, xr, R, mx = oracle.ref_imats_linearsolve(n, 1, A, b)
    assert st == 0
    exact = _rational_solve(M, bb)
    for i in range(n):
        assert Fraction(xr[2 * i]) <= exact[i] <= Fraction(xr[2 * i + 1])


def _rational_solve(M, b):
    """Exact solution of M x = b (integer entries) by Gaussian elimination
    over the rationals."""
    n = len(b)
    a = [[Fraction(int(M[i, j])) for j in range(n)] + [Fraction(int(b[i]))] for i in range(n)]
    for c in range(n):
        p = next(r for r in range(c, n) if a[r][c] != 0)
        a[c], a[p] = a[p], a[c]
        for r in range(n):
            if r != c and a[r][c] != 0:
                f = a[r][c] / a[c][c]
                a[r] = [x - f * y for x, y in zip(a[r], a[c])]
    return [a[i][n] / a[i][i] for i in range(n)]


def test_oracle_eigsymge_matches_golden(oracle, golden):
    """imats::eigsymge's verification (restated) on the reference's own X,
    lambda, Y: every bit of the merged enclosures."""
    for idx in range(int(golden["n_ge"][0])):
        n = int(golden[f"ge{idx}_n"][0])
        st, lam, bound = oracle.ieigsymge(n, golden[f"ge{idx}_A"], golden[f"ge{idx}_B"],
                                          golden[f"ge{idx}_X"], golden[f"ge{idx}_lambda"],
                                          golden[f"ge{idx}_Y"])
        assert st == 0 and bound == float(golden[f"ge{idx}_bound"][0]), idx
        assert np.array_equal(bits(lam), bits(golden[f"ge{idx}_lam"])), idx


def test_oracle_eigsymge_matches_reference_build(oracle):
    """Live: the reference's imats<double, pidblas>::eigsymge (project-written
    dsygv for its LAPACK call) against the restatement on its X, lambda, Y,
    including its base-class kv loops and the overlap merge."""
    if oracle.ref_lib() is None:
        from oracle.build import build_reference
        if build_reference() is None:
            pytest.skip("reference sources not mounted")
    rng = np.random.default_rng(41)
    for n, rel in [(3, 2.0 ** -30), (9, 2.0 ** -20), (25, 2.0 ** -36), (33, 2.0 ** -10)]:
        Am = rng.standard_normal((n, n))
        Am = (Am + Am.T) / 2
        if n == 9:  # a repeated eigenvalue: overlapping enclosures get merged
            Am = np.diag(np.repeat([1.0, 2.0, 3.0], 3))
        Bm = np.eye(n) + 0.05 * rng.standard_normal((n, n))
        Bm = Bm @ Bm.T
        A = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * rel)
        B = W._kv(Bm.ravel(order="F"), np.abs(Bm.ravel(order="F")) * rel)
        st, lam_r, X, lmb, Y = oracle.ref_imats_eigsymge(n, A, B)
        st2, lam_o, _ = oracle.ieigsymge(n, A, B, X, lmb, Y)
        assert st == st2 == 0, n
        assert np.array_equal(bits(lam_o), bits(lam_r)), n


def test_oracle_pddblas_matches_golden(oracle, golden):
    """pddblas::mulmm / mulltmm restated (oracle/vcp_oracle.c) against the
    reference's own products (golden vectors, scalar shortcuts included)."""
    for idx in range(int(golden["n_dd"][0])):
        m, n, k = (int(x) for x in golden[f"dd{idx}_shape"])
        A, B = golden[f"dd{idx}_A"], golden[f"dd{idx}_B"]
        C = oracle.pddblas_mulmm(m, n, k, A, B)
        assert np.array_equal(C.view(np.int64), golden[f"dd{idx}_C"].view(np.int64)), idx
        T = oracle.pddblas_mulltmm(k, n, B)
        assert np.array_equal(T.view(np.int64), golden[f"dd{idx}_T"].view(np.int64)), idx


def test_oracle_pddblas_matches_reference_build(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("reference build absent")
    rng = np.random.default_rng(31)
    for (m, n, k, phi) in [(17, 13, 70, 8), (64, 3, 900, 0), (2, 2, 5000, 32)]:
        hi = lambda r, c: rng.uniform(1, 2, r * c) * np.ldexp(1.0, rng.integers(-phi, phi + 1, r * c))  # noqa: E731
        def dd(r, c):
            h = hi(r, c) * rng.choice([-1.0, 1.0], r * c)
            out = np.empty(2 * r * c)
            out[0::2], out[1::2] = h, h * 2.0 ** -53 * rng.uniform(-1, 1, r * c)
            return out
        A, B = dd(m, k), dd(k, n)
        C = oracle.pddblas_mulmm(m, n, k, A, B)
        assert np.array_equal(C.view(np.int64), oracle.ref_pddblas_mulmm(m, n, k, A, B).view(np.int64))
        T = oracle.pddblas_mulltmm(k, n, B)
        assert np.array_equal(T.view(np.int64), oracle.ref_pddblas_mulltmm(k, n, B).view(np.int64))
