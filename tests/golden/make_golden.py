"""Generate the golden vectors in tests/golden/ from the reference itself.

The reference ships no golden vectors (its tests are print-only mains), so
this script runs the reference's own code -- vblas rmatmul,
vcp::matrix<kv::interval<double>, vcp::pidblas> and
vcp::matrix<kv::dd, vcp::pddblas> compiled from the reference tree by
oracle/build.py (kv from the project's kvshim) -- on small seeded
inputs and stores inputs and outputs as golden.npz.  It needs the reference
sources, so it runs only where they are mounted; the .npz travels with the
repository.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from oracle.build import build_reference  # noqa: E402
from vcp_gb300 import workloads as W  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"


def mixed_intervals(rng, n: int) -> np.ndarray:
    """kv buffer of n intervals of every sign case of vcp::ifma: positive,
    negative, straddling zero, [0, 0] and [0, x]."""
    a = rng.standard_normal(n)
    b = rng.standard_normal(n)
    lo, up = np.minimum(a, b), np.maximum(a, b)
    kind = rng.integers(0, 4, n)
    pos, neg, zer = kind == 1, kind == 2, kind == 3
    lo[pos] = np.abs(lo[pos])
    up[pos] = lo[pos] + np.abs(up[pos])
    up[neg] = -np.abs(up[neg])
    lo[neg] = up[neg] - np.abs(lo[neg])
    lo[zer] = 0.0
    up[zer] = np.where(rng.random(int(zer.sum())) < 0.5, 0.0, np.abs(up[zer]))
    out = np.empty(2 * n)
    out[0::2], out[1::2] = lo, up
    return out


def dd_matrix(rng, rows: int, cols: int, phi: int) -> np.ndarray:
    """kv::dd pairs (column-major): hi from E(phi), lo = hi 2^-53 u, u in [-1, 1]."""
    hi = W.ephi(rng, rows * cols, phi)
    out = np.empty(2 * rows * cols)
    out[0::2] = hi
    out[1::2] = hi * 2.0 ** -53 * rng.uniform(-1.0, 1.0, rows * cols)
    return out


def main() -> None:
    if build_reference() is None:
        raise SystemExit("reference sources not mounted; cannot regenerate golden vectors")
    rng = np.random.default_rng(20261203)
    data: dict[str, np.ndarray] = {}
    # vblas rmatmul, vblas naming (A m x n, B n x k), three modes, ragged shapes
    cases = [(1, 1, 1), (7, 5, 3), (16, 64, 4), (33, 17, 29), (64, 64, 64), (3, 200, 2)]
    for idx, (m, n, k) in enumerate(cases):
        phi = [0, 8, 32][idx % 3]
        A = W.ephi(rng, m * n, phi)
        B = W.ephi(rng, n * k, phi)
        data[f"rm{idx}_shape"] = np.array([m, n, k])
        data[f"rm{idx}_A"] = A
        data[f"rm{idx}_B"] = B
        for rnd, tag in ((1, "up"), (-1, "dn"), (0, "rn")):
            data[f"rm{idx}_{tag}"] = O.ref_rmatmul(m, n, k, A, B, rnd)
    # pidblas::mulmm through vcp::matrix, GEMM naming (A m x k, B k x n)
    icases = [(5, 4, 6), (32, 32, 32), (17, 40, 64), (64, 9, 3)]
    for idx, (m, n, k) in enumerate(icases):
        A = W.interval_ephi(rng, m, k, phi=4, rad_ratio=2.0 ** -40)
        B = W.interval_ephi(rng, k, n, phi=4, rad_ratio=2.0 ** -20)
        data[f"iv{idx}_shape"] = np.array([m, n, k])
        data[f"iv{idx}_A"] = A
        data[f"iv{idx}_B"] = B
        data[f"iv{idx}_C"] = O.ref_pidblas_mulmm(m, n, k, A, B)
    # pidblas::mul_im_m / mul_m_im, mulltmm, vmulmm and the linearsolve bound
    import ctypes
    pcases = [(0, 9, 7, 11), (1, 9, 7, 11), (0, 33, 20, 64), (1, 20, 33, 64)]
    for idx, (side, m, n, k) in enumerate(pcases):
        L = W.interval_ephi(rng, m, k, 4, 2.0 ** -30) if side == 0 else W.ephi(rng, m * k, 4)
        R = W.ephi(rng, k * n, 4) if side == 0 else W.interval_ephi(rng, k, n, 4, 2.0 ** -30)
        C = np.zeros(2 * m * n)
        assert O.ref_call("ref_pidblas_mul_point", side, m, n, k, O._p(L), O._p(R), O._p(C)) == 0
        data[f"mp{idx}_shape"] = np.array([side, m, n, k])
        data[f"mp{idx}_L"], data[f"mp{idx}_R"], data[f"mp{idx}_C"] = L, R, C
    for idx, (n, k) in enumerate([(6, 9), (40, 33)]):
        A = W.interval_ephi(rng, k, n, 4, 2.0 ** -20)
        C = np.zeros(2 * n * n)
        assert O.ref_call("ref_pidblas_mulltmm", n, k, O._p(A), O._p(C)) == 0
        P = W.ephi(rng, k * n, 8)
        V = np.zeros(2 * n * n)
        assert O.ref_call("ref_pidblas_vmulmm", n, k, O._p(P), O._p(V)) == 0
        data[f"sy{idx}_shape"] = np.array([n, k])
        data[f"sy{idx}_A"], data[f"sy{idx}_C"] = A, C
        data[f"sy{idx}_P"], data[f"sy{idx}_V"] = P, V
    for idx, nn in enumerate([12, 48]):
        Am = np.eye(nn) + 0.05 * rng.standard_normal((nn, nn))
        Ai = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * 1e-9)
        Rinv = np.linalg.inv(Am).ravel(order="F")
        g = ctypes.c_double(0.0)
        assert O.ref_call("ref_norm_I_minus_RA", nn, O._p(Rinv), O._p(Ai), ctypes.addressof(g)) == 0
        data[f"nm{idx}_n"] = np.array([nn])
        data[f"nm{idx}_R"], data[f"nm{idx}_A"] = Rinv, Ai
        data[f"nm{idx}_bound"] = np.array([g.value])
    # vcp::ifma elementwise and vcp::pidblas_fma::mulmm (own seed, so the
    # vectors above stay as they were)
    rng2 = np.random.default_rng(20261204)
    n_if = 4096
    A, B, Cc = (mixed_intervals(rng2, n_if) for _ in range(3))
    R = np.empty(2 * n_if)
    O.ref_lib().ref_ifma(n_if, O._p(A), O._p(B), O._p(Cc), O._p(R))
    data["if_A"], data["if_B"], data["if_C"], data["if_R"] = A, B, Cc, R
    fcases = [(5, 4, 6), (33, 17, 40), (64, 64, 20)]
    for idx, (m, n, k) in enumerate(fcases):
        A = mixed_intervals(rng2, m * k)
        B = mixed_intervals(rng2, k * n)
        C_ = np.empty(2 * m * n)
        assert O.ref_lib().ref_pidblas_fma_mulmm(m, n, k, O._p(A), O._p(B), O._p(C_)) == 0
        data[f"fm{idx}_shape"] = np.array([m, n, k])
        data[f"fm{idx}_A"], data[f"fm{idx}_B"], data[f"fm{idx}_C"] = A, B, C_
    # imats<double, pidblas>::linearsolve (own seed again): inputs, the R and
    # mx it works with, its enclosure x and the bound ||RA - I||; the last
    # case fails the check (the reference throws, status 2)
    rng3 = np.random.default_rng(20261205)
    lcases = [(2, 1, 2.0 ** -30), (16, 1, 2.0 ** -30), (33, 3, 2.0 ** -24), (48, 1, 2.0 ** -40),
              (64, 5, 2.0 ** -30), (8, 1, 0.5)]
    for idx, (n, nrhs, rel) in enumerate(lcases):
        Am = rng3.uniform(-1.0, 1.0, (n, n)) + (2.0 if rel > 0.1 else 4.0) * np.eye(n)
        A = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * rel)
        bm = rng3.uniform(-1.0, 1.0, n * nrhs)
        b = W._kv(bm, np.abs(bm) * 2.0 ** -35)
        st, x, R, mx = O.ref_imats_linearsolve(n, nrhs, A, b)
        g = ctypes.c_double(0.0)
        assert O.ref_call("ref_norm_I_minus_RA", n, O._p(R), O._p(A), ctypes.addressof(g)) == 0
        data[f"ls{idx}_shape"] = np.array([n, nrhs])
        data[f"ls{idx}_A"], data[f"ls{idx}_b"] = A, b
        data[f"ls{idx}_R"], data[f"ls{idx}_mx"], data[f"ls{idx}_x"] = R, mx, x
        data[f"ls{idx}_status"] = np.array([st])
        data[f"ls{idx}_bound"] = np.array([g.value])
    data["n_ls"] = np.array([len(lcases)])
    # imats<double, pidblas>::eigsymge (own seed): A, B symmetric, mid B
    # positive definite; the X, lambda, Y it works with and its enclosures
    rng4 = np.random.default_rng(20261207)
    gcases = [(2, 2.0 ** -30), (6, 2.0 ** -40), (17, 2.0 ** -30), (40, 2.0 ** -24)]
    for idx, (n, rel) in enumerate(gcases):
        Am = rng4.standard_normal((n, n))
        Am = (Am + Am.T) / 2
        Bm = np.eye(n) + 0.1 * rng4.standard_normal((n, n))
        Bm = Bm @ Bm.T
        A = W._kv(Am.ravel(order="F"), np.abs(Am.ravel(order="F")) * rel)
        B = W._kv(Bm.ravel(order="F"), np.abs(Bm.ravel(order="F")) * rel)
        st, lam, X, lmb, Y = O.ref_imats_eigsymge(n, A, B)
        assert st == 0
        _, _, bound = O.ieigsymge(n, A, B, X, lmb, Y)
        data[f"ge{idx}_n"] = np.array([n])
        data[f"ge{idx}_A"], data[f"ge{idx}_B"] = A, B
        data[f"ge{idx}_X"], data[f"ge{idx}_lambda"], data[f"ge{idx}_Y"] = X, lmb, Y
        data[f"ge{idx}_lam"] = lam
        data[f"ge{idx}_bound"] = np.array([bound])
    # pddblas::mulmm / mulltmm (the dd Ozaki products, vcp/pddblas.hpp:318-409)
    # through vcp::matrix<kv::dd, vcp::pddblas>: hi words E(phi), lo = hi 2^-53 u
    rng5 = np.random.default_rng(20261208)
    dcases = [(1, 1, 1, 0), (1, 7, 1, 3), (6, 1, 1, 2), (9, 7, 13, 0), (20, 12, 300, 16),
              (6, 5, 2100, 4)]
    for idx, (m, n, k, phi) in enumerate(dcases):
        A = dd_matrix(rng5, m, k, phi)
        B = dd_matrix(rng5, k, n, phi)
        data[f"dd{idx}_shape"] = np.array([m, n, k])
        data[f"dd{idx}_A"], data[f"dd{idx}_B"] = A, B
        data[f"dd{idx}_C"] = O.ref_pddblas_mulmm(m, n, k, A, B)
        data[f"dd{idx}_T"] = O.ref_pddblas_mulltmm(k, n, B)
    data["n_dd"] = np.array([len(dcases)])
    # pddblas's refinement consumers (vcp/pddblas.hpp:413-563) as the
    # reference runs them: linearsolve, inv, Cholesky on well-conditioned
    # dd matrices (LU / Cholesky / triangular solves project-written)
    import ctypes
    R = O.ref_lib()
    R.ref_pddblas_linearsolve.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 3
    R.ref_pddblas_unary.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 2
    rng6 = np.random.default_rng(20261209)
    lcases = [(12, 1), (40, 3)]
    for idx, (n, nrhs) in enumerate(lcases):
        A = dd_matrix(rng6, n, n, 2)
        A[0::2][np.arange(n) * (n + 1)] += 4.0 * n   # diagonally dominant
        b = dd_matrix(rng6, n, nrhs, 2)
        x = np.empty(2 * n * nrhs)
        assert R.ref_pddblas_linearsolve(n, nrhs, A.ctypes.data, b.ctypes.data, x.ctypes.data) == 0
        data[f"pls{idx}_shape"] = np.array([n, nrhs])
        data[f"pls{idx}_A"], data[f"pls{idx}_b"], data[f"pls{idx}_x"] = A, b, x
    data["n_pls"] = np.array([len(lcases)])
    n = 16
    A = dd_matrix(rng6, n, n, 1)
    A[0::2][np.arange(n) * (n + 1)] += 3.0 * n
    Ri = np.empty(2 * n * n)
    assert R.ref_pddblas_unary(0, n, A.ctypes.data, Ri.ctypes.data) == 0
    data["inv_n"], data["inv_A"], data["inv_R"] = np.array([n]), A, Ri
    n = 24
    G = dd_matrix(rng6, n, n, 1)
    Gm = G[0::2].reshape(n, n, order="F")
    S = Gm @ Gm.T + n * np.eye(n)
    Sd = np.empty(2 * n * n)
    Sd[0::2] = S.ravel(order="F")
    lo = (S * 2.0 ** -53 * rng6.uniform(-1, 1, (n, n)))
    lo = np.triu(lo) + np.triu(lo, 1).T             # symmetric dd
    Sd[1::2] = lo.ravel(order="F")
    U = np.empty(2 * n * n)
    assert R.ref_pddblas_unary(1, n, Sd.ctypes.data, U.ctypes.data) == 0
    data["chol_n"], data["chol_A"], data["chol_U"] = np.array([n]), Sd, U
    # pddblas::eigsym / eigsymge with eigenvectors (Ogita-Aishima refinement
    # of the double eigenpairs; dsyev / dsygv project-written): symmetric
    # matrices with well separated eigenvalues
    R.ref_pddblas_eig.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                  ctypes.c_void_p, ctypes.c_void_p]

    def sym_dd(nn, spectrum):
        Qm, _ = np.linalg.qr(rng6.standard_normal((nn, nn)))
        S = (Qm * spectrum) @ Qm.T
        S = (S + S.T) / 2
        lo = S * 2.0 ** -53 * rng6.uniform(-1, 1, (nn, nn))
        lo = np.triu(lo) + np.triu(lo, 1).T
        out = np.empty(2 * nn * nn)
        out[0::2], out[1::2] = S.ravel(order="F"), lo.ravel(order="F")
        return out
    n = 20
    A = sym_dd(n, np.arange(1.0, n + 1.0) * 1.5)
    lam, X = np.empty(2 * n), np.empty(2 * n * n)
    assert R.ref_pddblas_eig(n, A.ctypes.data, None, 1, lam.ctypes.data, X.ctypes.data) == 0
    data["eig_n"], data["eig_A"], data["eig_lam"], data["eig_X"] = np.array([n]), A, lam, X
    n = 16
    A = sym_dd(n, np.linspace(-3.0, 5.0, n))
    B = sym_dd(n, np.linspace(1.0, 2.0, n))
    lam, X = np.empty(2 * n), np.empty(2 * n * n)
    assert R.ref_pddblas_eig(n, A.ctypes.data, B.ctypes.data, 1, lam.ctypes.data,
                             X.ctypes.data) == 0
    data["eigge_n"], data["eigge_A"], data["eigge_B"] = np.array([n]), A, B
    data["eigge_lam"], data["eigge_X"] = lam, X
    data["n_ge"] = np.array([len(gcases)])
    data["n_fm"] = np.array([len(fcases)])
    data["n_mp"] = np.array([len(pcases)])
    data["n_sy"] = np.array([2])
    data["n_nm"] = np.array([2])
    data["n_rm"] = np.array([len(cases)])
    data["n_iv"] = np.array([len(icases)])
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")
    write_vcpmat_fixtures()


def write_vcpmat_fixtures() -> None:
    """.vcpmat files written by the reference's own vcp::save_portable
    (tests/golden/vcpmat/): an interval product A (33 x 17) * B (17 x 20) = C
    from vcp::matrix<interval, pidblas>, and one small matrix of every other
    element type."""
    import ctypes
    R = O.ref_lib()
    R.ref_vcpmat_save.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_void_p]
    d = Path(__file__).resolve().parent / "vcpmat"
    d.mkdir(exist_ok=True)
    rng = np.random.default_rng(20261206)
    m, n, k = 33, 20, 17
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -30)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -20)
    C = O.ref_pidblas_mulmm(m, n, k, A, B)
    mats = [("A", 3, m, k, A), ("B", 3, k, n, B), ("C", 3, m, n, C),
            ("int32", 1, 5, 4, rng.integers(-1000, 1000, 20).astype(np.int32)),
            ("double", 2, 4, 6, W.ephi(rng, 24, 30)),
            ("dd", 4, 3, 5, np.ravel(np.stack([W.ephi(rng, 15, 3), W.ephi(rng, 15, 3) * 2.0 ** -60],
                                               axis=1))),
            ("interval_dd", 5, 2, 3, np.sort(W.ephi(rng, 24, 2)))]
    for name, kind, r, c, buf in mats:
        buf = np.ascontiguousarray(buf)
        assert R.ref_vcpmat_save(str(d / name).encode(), kind, r, c, buf.ctypes.data) == 0
    print(f"wrote {len(mats)} .vcpmat fixtures to {d}")


if __name__ == "__main__":
    main()
