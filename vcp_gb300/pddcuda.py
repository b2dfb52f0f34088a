"""Double-double GEMM with pddblas semantics on the GPU (the vcp::pddcuda policy).

dd matrices use the kv::dd memory layout: column-major, each entry a pair
{a1, a2} of doubles (value a1 + a2).  ``mulmm(A, B, m, n, k)`` returns the dd
product C (kv buffer) and a rigorous per-entry upper bound of |AB - C|
(vcp/pddblas.hpp:318-376 computes the same product, approximately, with
double slices and dd accumulation).  ``linearsolve``, ``inv``,
``cholesky``, ``eigsym`` and ``eigsymge`` are pddblas's refinement loops
with their products here.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .vblas import _dev_ptr, _host_ptr, _stream_ptr


def mulmm(A: np.ndarray, B: np.ndarray, m: int, n: int, k: int, slices: int = 0,
          with_bound: bool = True):
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    C = np.empty(2 * m * n, dtype=np.float64)
    E = np.empty(m * n, dtype=np.float64) if with_bound else None
    if m <= 0 or n <= 0:
        return C, E
    pa = _host_ptr(A, 2 * m * k, "A") if k > 0 else None
    pb = _host_ptr(B, 2 * k * n, "B") if k > 0 else None
    _lib.call("vcpcu_ddgemm", m, n, k, pa, pb, C.ctypes.data,
              E.ctypes.data if E is not None else None, int(slices))
    return C, E


def mulmm_dev(m, n, k, A, lda, B, ldb, C, ldc, Cerr=None, lde=0, slices=0, stream=None):
    _lib.call("vcpcu_ddgemm_dev", m, n, k, _dev_ptr(A, "A"), lda, _dev_ptr(B, "B"), ldb,
              _dev_ptr(C, "C"), ldc, _dev_ptr(Cerr, "Cerr") if Cerr is not None else None,
              lde, int(slices), _stream_ptr(stream))


def mulltmm(A: np.ndarray, n: int, k: int, slices: int = 0):
    """A^T A for a dd A (k x n), as pddblas::mulltmm (vcp/pddblas.hpp:379-409)."""
    At = A.reshape(n, k, 2).transpose(1, 0, 2).copy().reshape(-1)
    C, E = mulmm(At, A, n, n, k, slices)
    Cm = C.reshape(n, n, 2)
    Em = E.reshape(n, n)
    iu = np.triu_indices(n, 1)
    # enforce exact symmetry from the upper triangle, as pddblas does
    Cm[iu[0], iu[1]] = Cm[iu[1], iu[0]]
    Em[iu[0], iu[1]] = Em[iu[1], iu[0]]
    return C, E


# ---- the refinement consumers of pddblas (vcp/pddblas.hpp:413-563) ----------------
#
# pddblas's linear solve, inverse and Cholesky factor run their approximate
# steps in double (LAPACK) and every accurate residual through the Ozaki
# product (pddblas_assist::ozaki_acc).  These are the same loops with each
# such product on the GPU (vcpcu_ddgemm) and the dd arithmetic of the kv
# type, elementwise in numpy (round to nearest: TwoSum, Dekker's
# renormalisation).  The C++ drop-in (include/vcp_cuda/pddcuda.hpp) runs the
# same loops behind vcp::matrix<kv::dd, vcp::pddcuda>.

def _twosum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _fasttwosum(a, b):
    s = a + b
    return s, b - (s - a)


def dd_add(x1, x2, y1, y2):
    """x + y for dd arrays (kv::dd addition: TwoSum of both words, two
    renormalisations)."""
    s, e = _twosum(x1, y1)
    t, f = _twosum(x2, y2)
    e = e + t
    s, e = _fasttwosum(s, e)
    e = e + f
    return _fasttwosum(s, e)


def _kv(hi, lo):
    out = np.empty(2 * hi.size, dtype=np.float64)
    out[0::2] = hi.ravel(order="F")
    out[1::2] = lo.ravel(order="F")
    return out


def _words(X, rows, cols):
    return (X[0::2].reshape(rows, cols, order="F").copy(),
            X[1::2].reshape(rows, cols, order="F").copy())


def linearsolve(A: np.ndarray, b: np.ndarray, n: int, nrhs: int, slices: int = 0,
                itmax: int = 10) -> np.ndarray:
    """x = A \\ b for dd A (n x n) and b (n x nrhs), kv buffers, as
    pddblas::linearsolve (vcp/pddblas.hpp:413-474): LU of double(A), then up
    to itmax corrections d = LU \\ double(r), x += d, r = b - A x with A x
    the dd product on the GPU; stops at dd accuracy (|d| <= 0.25e-32 |x|) or
    when a correction fails to halve.  Returns the kv buffer of x."""
    import scipy.linalg
    Ah, _ = _words(A, n, n)
    lu = scipy.linalg.lu_factor(Ah)
    bh, bl = _words(b, n, nrhs)
    xh = np.zeros((n, nrhs))
    xl = np.zeros((n, nrhs))
    rh, rl = bh.copy(), bl.copy()
    prev = np.inf
    for _ in range(itmax):
        d = scipy.linalg.lu_solve(lu, rh)
        xh, xl = dd_add(xh, xl, d, np.zeros_like(d))
        normd = float(np.max(np.abs(d))) if d.size else 0.0
        normx = float(np.max(np.abs(xh))) if xh.size else 0.0
        if normd == 0.0 or normd <= 0.25e-32 * normx or normd >= 0.5 * prev:
            break
        prev = normd
        Ax, _ = mulmm(A, _kv(xh, xl), n, nrhs, n, slices, with_bound=False)
        axh, axl = _words(Ax, n, nrhs)
        rh, rl = dd_add(bh, bl, -axh, -axl)
    return _kv(xh, xl)


def inv(A: np.ndarray, n: int, slices: int = 0) -> np.ndarray:
    """inv(A) for a dd A (pddblas::inv, vcp/pddblas.hpp:477-486): A X = I by
    linearsolve."""
    eye = _kv(np.eye(n), np.zeros((n, n)))
    return linearsolve(A, eye, n, n, slices)


def cholesky(A: np.ndarray, n: int, slices: int = 0, itep: int = 2) -> np.ndarray:
    """Upper Cholesky factor U (A = U^T U) of a symmetric dd A, as
    pddblas::Cholesky (vcp/pddblas.hpp:490-563): U from the double factor,
    then itep refinements E = A - U^T U (dd product on the GPU),
    G = U^-T E U^-1 in double, W = triu(G, 1) + diag(G) / 2, U += W U
    (GPU); the entries below the diagonal exact zeros."""
    import scipy.linalg
    Ah, Al = _words(A, n, n)
    Ud = scipy.linalg.cholesky(Ah, lower=False)   # dpotrf "U", lower triangle zero
    uh, ul = Ud.copy(), np.zeros((n, n))
    for _ in range(itep):
        U = _kv(uh, ul)
        Ut = _kv(uh.T.copy(), ul.T.copy())
        UtU, _ = mulmm(Ut, U, n, n, n, slices, with_bound=False)
        th, tl = _words(UtU, n, n)
        eh, el = dd_add(Ah, Al, -th, -tl)
        Udh = uh
        G = scipy.linalg.solve_triangular(Udh, eh, trans="T", lower=False)   # U^-T E
        G = scipy.linalg.solve_triangular(Udh, G.T, trans="T", lower=False).T  # ... U^-1
        W = np.triu(G, 1) + np.diag(np.diag(G)) * 0.5
        F, _ = mulmm(_kv(W, np.zeros((n, n))), U, n, n, n, slices, with_bound=False)
        fh, fl = _words(F, n, n)
        uh, ul = dd_add(uh, ul, fh, fl)
    il = np.tril_indices(n, -1)
    uh[il] = 0.0
    ul[il] = 0.0
    return _kv(uh, ul)


def _split(a):
    c = 134217729.0 * a          # Veltkamp splitting, 2^27 + 1
    hi = c - (c - a)
    return hi, a - hi


def _twoprod(a, b):
    """p + e = a b exactly (Dekker)."""
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    return p, ((ah * bh - p) + ah * bl + al * bh) + al * bl


def dd_mul(x1, x2, y1, y2):
    """x y for dd arrays (the kv stand-in's product: TwoProduct of the
    leading words plus the cross terms, renormalised)."""
    p, e = _twoprod(x1, y1)
    e = e + (x1 * y2 + x2 * y1)
    return _fasttwosum(p, e)


def dd_div(x1, x2, y1, y2):
    """x / y for dd arrays: the leading quotient and one correction from the
    dd remainder x - y q1."""
    q1 = x1 / y1
    t1, t2 = dd_mul(y1, y2, q1, np.zeros_like(q1))
    r1, _ = dd_add(x1, x2, -t1, -t2)
    return _fasttwosum(q1, r1 / y1)


def _oa_step(A, B, xh, xl, n, slices):
    """One Ogita-Aishima refinement step (pddblas::oa_step,
    vcp/pddblas.hpp:221-314) for A x = lambda B x (B None: B = I), every
    product on the GPU.  Returns the refined X and the eigenvalues."""
    X = _kv(xh, xl)
    Xt = _kv(xh.T.copy(), xl.T.copy())
    AX, _ = mulmm(A, X, n, n, n, slices, with_bound=False)
    S, _ = mulmm(Xt, AX, n, n, n, slices, with_bound=False)
    if B is not None:
        BX, _ = mulmm(B, X, n, n, n, slices, with_bound=False)
        G, _ = mulmm(Xt, BX, n, n, n, slices, with_bound=False)
    else:
        G, _ = mulmm(Xt, X, n, n, n, slices, with_bound=False)
    sh, sl = _words(S, n, n)
    gh, gl = _words(G, n, n)
    d = np.arange(n)
    lh, ll = dd_div(sh[d, d], sl[d, d], gh[d, d], gl[d, d])   # lambda_i = S_ii / G_ii
    rh, rl = -gh, -gl                                          # R = I - G
    rh[d, d], rl[d, d] = dd_add(rh[d, d], rl[d, d], np.ones(n), np.zeros(n))
    normR = float(np.max(np.sum(np.abs(rh), axis=1)))
    offS = float(np.max(np.sum(np.abs(sh), axis=1) - np.abs(sh[d, d])))
    delta = 2.0 * (offS + normR * float(np.max(np.abs(lh))))
    # E_ij = (S_ij + lambda_j R_ij) / (lambda_j - lambda_i) where separated,
    # R_ij / 2 otherwise (and on the diagonal)
    Lj1, Lj2 = np.broadcast_to(lh, (n, n)), np.broadcast_to(ll, (n, n))
    Li1, Li2 = np.broadcast_to(lh[:, None], (n, n)), np.broadcast_to(ll[:, None], (n, n))
    dh, dl = dd_add(Lj1, Lj2, -Li1, -Li2)
    nh, nl = dd_add(sh, sl, *dd_mul(Lj1, Lj2, rh, rl))
    with np.errstate(divide="ignore", invalid="ignore"):   # unseparated pairs: not used
        qh, ql = dd_div(nh, nl, dh, dl)
    sep = (np.abs(dh) > delta) & ~np.eye(n, dtype=bool)
    eh = np.where(sep, qh, rh * 0.5)
    el = np.where(sep, ql, rl * 0.5)
    XE, _ = mulmm(X, _kv(eh, el), n, n, n, slices, with_bound=False)
    fh, fl = _words(XE, n, n)
    xh, xl = dd_add(xh, xl, fh, fl)
    return xh, xl, lh, ll


def eigsym(A: np.ndarray, n: int, itep: int = 1, slices: int = 0, B: np.ndarray | None = None):
    """Eigenvalues and eigenvectors of a symmetric dd A (B None) or of
    A x = lambda B x, as pddblas::eigsym / eigsymge (vcp/pddblas.hpp:566-657):
    the double eigenpairs of LAPACK (dsyev / dsygv), then max(2, itep)
    Ogita-Aishima steps with their products on the GPU.  Returns (lambda as
    a kv buffer of n dd values, X as a kv buffer of n x n, columns the
    eigenvectors)."""
    import scipy.linalg
    Ah, _ = _words(A, n, n)
    if B is None:
        w, V = scipy.linalg.eigh(Ah)
    else:
        Bh, _ = _words(B, n, n)
        w, V = scipy.linalg.eigh(Ah, Bh)
    xh, xl = np.array(V, dtype=np.float64, order="C"), np.zeros((n, n))
    lh, ll = np.asarray(w, dtype=np.float64), np.zeros(n)
    for _ in range(max(2, itep)):
        xh, xl, lh, ll = _oa_step(A, B, xh, xl, n, slices)
    lam = np.empty(2 * n)
    lam[0::2], lam[1::2] = lh, ll
    return lam, _kv(xh, xl)


def eigsymge(A: np.ndarray, B: np.ndarray, n: int, itep: int = 1, slices: int = 0):
    """A x = lambda B x for symmetric dd A, B (pddblas::eigsymge)."""
    return eigsym(A, n, itep, slices, B=B)
