"""ctypes front end of the CPU oracle (liboracle.so) and of the reference
build (oracle/_ref/libvcpref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, as the checker or the timed CPU baseline.  The
product (vcp_gb300, libvcpcuda.so) never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import LIB, REF_LIB, build_oracle

_i, _l, _v = C.c_int, C.c_long, C.c_void_p
_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(str(LIB))
        L.orc_rmatmul.argtypes = [_i, _i, _i, _v, _v, _v, _i, _i]
        L.orc_rmatmul_ld.argtypes = [_i, _i, _i, _v, _l, _v, _l, _v, _l, _i, _i]
        L.orc_udmatmul.argtypes = [_i, _i, _i, _v, _v, _v, _v, _i]
        L.orc_midrad.argtypes = [_l, _v, _v, _v]
        L.orc_pidblas_mulmm.argtypes = [_i, _i, _i, _v, _v, _v, _i]
        L.orc_exact_hull.argtypes = [_i, _i, _i, _v, _v, _l, _v, _v, _v, _v, _i]
        L.orc_exact_dot.argtypes = [_i, _i, _i, _v, _v, _l, _v, _v, _v, _v, _i]
        L.orc_exact_sum.argtypes = [_l, _v, _i]
        L.orc_ifma.argtypes = [_l, _v, _v, _v, _v]
        L.orc_pidblas_fma_mulmm.argtypes = [_i, _i, _i, _v, _v, _v, _i]
        L.orc_dd_residual.argtypes = [_i, _i, _i, _v, _v, _v, _l, _v, _v, _v, _v, _i]
        L.orc_exact_sum.restype = C.c_double
        L.orc_ozaki_igemm.argtypes = [_i, _i, _i, _v, _v, _v, _i, _i]
        L.orc_ozaki_igemm.restype = _i
        L.orc_ozaki2_igemm.argtypes = [_i, _i, _i, _v, _v, _v, _i, _i]
        L.orc_ozaki2_igemm.restype = _i
        L.orc_pidblas_mul_point.argtypes = [_i, _i, _i, _i, _v, _v, _v, _i]
        L.orc_pidblas_mul_point.restype = _i
        L.orc_pidblas_mulltmm.argtypes = [_i, _i, _v, _v, _i]
        L.orc_pidblas_mulltmm.restype = _i
        L.orc_pidblas_vmulmm.argtypes = [_i, _i, _v, _v, _i]
        L.orc_pidblas_vmulmm.restype = _i
        L.orc_norm_I_minus_RA.argtypes = [_i, _v, _v, _i]
        L.orc_norm_I_minus_RA.restype = C.c_double
        L.orc_ilss_verify.argtypes = [_i, _i, _v, _v, _v, _v, _v, _v, _v, _i]
        L.orc_ilss_verify.restype = _i
        L.orc_ieigsymge.argtypes = [_i, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v, _i, _i]
        L.orc_ieigsymge.restype = _i
        L.orc_imats_mul_m_im_naive.argtypes = [_i, _i, _i, _v, _v, _v]
        L.orc_eig_merge.argtypes = [_i, _v]
        L.orc_tensor_basis.argtypes = [_i, _v, _v, _i, _v, _v, _i, _i, _v, _v, _v, _l, _i, _i,
                                       _i]
        L.orc_tensor_basis.restype = _i
        L.orc_pddblas_mulmm.argtypes = [_i, _i, _i, _v, _v, _v, _i]
        L.orc_pddblas_mulmm.restype = _i
        L.orc_pddblas_mulltmm.argtypes = [_i, _i, _v, _v, _i]
        L.orc_pddblas_mulltmm.restype = _i
        L.orc_fp64_peak.argtypes = [C.c_double, _i]
        L.orc_fp64_peak.restype = C.c_double
        _lib = L
    return _lib


def ref_lib() -> C.CDLL | None:
    """The reference compiled from its own sources, or None where absent."""
    global _ref
    if _ref is None and Path(REF_LIB).exists():
        R = C.CDLL(str(REF_LIB))
        R.ref_rmatmul.argtypes = [_i, _i, _i, _v, _v, _v, _i]
        R.ref_pidblas_mulmm.argtypes = [_i, _i, _i, _v, _v, _v]
        R.ref_pidblas_mulmm.restype = _i
        R.ref_pidblas_mul_point.argtypes = [_i, _i, _i, _i, _v, _v, _v]
        R.ref_pidblas_mul_point.restype = _i
        R.ref_pidblas_mulltmm.argtypes = [_i, _i, _v, _v]
        R.ref_pidblas_mulltmm.restype = _i
        R.ref_pidblas_vmulmm.argtypes = [_i, _i, _v, _v]
        R.ref_pidblas_vmulmm.restype = _i
        R.ref_norm_I_minus_RA.argtypes = [_i, _v, _v, _v]
        R.ref_ifma.argtypes = [_l, _v, _v, _v, _v]
        R.ref_pidblas_fma_mulmm.argtypes = [_i, _i, _i, _v, _v, _v]
        R.ref_pidblas_fma_mulmm.restype = _i
        R.ref_norm_I_minus_RA.restype = _i
        R.ref_pddblas_mulmm.argtypes = [_i, _i, _i, _v, _v, _v]
        R.ref_pddblas_mulmm.restype = _i
        R.ref_pddblas_mulltmm.argtypes = [_i, _i, _v, _v]
        R.ref_pddblas_mulltmm.restype = _i
        R.ref_imats_linearsolve.argtypes = [_i, _i, _v, _v, _v, _v, _v]
        R.ref_imats_linearsolve.restype = _i
        R.ref_imats_eigsymge.argtypes = [_i, _v, _v, _v, _v, _v, _v]
        R.ref_imats_eigsymge.restype = _i
        _ref = R
    return _ref


def _p(a: np.ndarray) -> int:
    assert a.dtype == np.float64 or a.dtype == np.int32
    assert a.flags.c_contiguous or a.flags.f_contiguous
    return a.ctypes.data


def rmatmul(m, n, k, A, B, rnd, threads=0) -> np.ndarray:
    """vblas naming (A m x n, B n x k); returns C (flat, column-major)."""
    C_ = np.zeros(max(m * k, 1), dtype=np.float64)
    lib().orc_rmatmul(m, n, k, _p(A), _p(B), _p(C_), int(rnd), int(threads))
    return C_


def pidblas_mulmm(m, n, k, A, B, threads=0) -> np.ndarray:
    """GEMM naming, kv-layout buffers; returns C's kv buffer."""
    C_ = np.zeros(2 * m * n, dtype=np.float64)
    st = lib().orc_pidblas_mulmm(m, n, k, _p(A), _p(B), _p(C_), int(threads))
    assert st == 0
    return C_


def midrad(X: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    cnt = X.size // 2
    m = np.empty(cnt)
    r = np.empty(cnt)
    lib().orc_midrad(cnt, _p(X), _p(m), _p(r))
    return m, r


def exact_hull(m, n, k, A, B, rows, cols, threads=0):
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    lo = np.empty(rows.size)
    up = np.empty(rows.size)
    lib().orc_exact_hull(m, n, k, _p(A), _p(B), rows.size, _p(rows), _p(cols), _p(lo), _p(up),
                         int(threads))
    return lo, up


def exact_dot(m, n, k, A, B, rows, cols, threads=0):
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    dn = np.empty(rows.size)
    up = np.empty(rows.size)
    lib().orc_exact_dot(m, n, k, _p(A), _p(B), rows.size, _p(rows), _p(cols), _p(dn), _p(up),
                        int(threads))
    return dn, up


def dd_residual(m, n, k, A, B, C, rows, cols, threads=0):
    """(RU|exact - C|, RD|exact|) per sampled entry of a dd product C ~ A B
    (dd pairs, ld = rows): the error of a dd GEMM against the exact value."""
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    err = np.empty(rows.size)
    ab = np.empty(rows.size)
    lib().orc_dd_residual(m, n, k, _p(A), _p(B), _p(C), rows.size, _p(rows), _p(cols), _p(err),
                          _p(ab), int(threads))
    return err, ab


def ozaki_igemm(m, n, k, A, B, s=8, sr=2, crt=True):
    """Host model of the Ozaki-form interval product (kv buffers, GEMM
    naming): crt=True the CRT form (GPU form OZAKI), crt=False the slice form
    (GPU form OZAKI_SLICES).  s may carry the fast-radius flag 0x100 (as
    the GPU form's slices argument).  Returns (C kv buffer, status) --
    status 3 on non-finite input."""
    C_ = np.zeros(2 * m * n, dtype=np.float64)
    fn = lib().orc_ozaki2_igemm if crt else lib().orc_ozaki_igemm
    st = fn(m, n, k, _p(A) if k > 0 else None, _p(B) if k > 0 else None, _p(C_), int(s), int(sr))
    return C_, st


def pidblas_mul_point(side, m, n, k, L, R, threads=0):
    """pidblas::mul_im_m (side 0: [L] R) / mul_m_im (side 1: L [R]); kv C."""
    C_ = np.zeros(2 * m * n)
    assert lib().orc_pidblas_mul_point(side, m, n, k, _p(L), _p(R), _p(C_), threads) == 0
    return C_


def pidblas_mulltmm(n, k, A, threads=0):
    C_ = np.zeros(2 * n * n)
    assert lib().orc_pidblas_mulltmm(n, k, _p(A), _p(C_), threads) == 0
    return C_


def pidblas_vmulmm(n, k, A, threads=0):
    C_ = np.zeros(2 * n * n)
    assert lib().orc_pidblas_vmulmm(n, k, _p(A), _p(C_), threads) == 0
    return C_


def norm_I_minus_RA(n, R, A, threads=0) -> float:
    return float(lib().orc_norm_I_minus_RA(n, _p(R), _p(A), threads))


def ilss_verify(n, nrhs, A, b, R, mx, E=None, threads=0):
    """imats::linearsolve's verification (restatement) for given R, mx:
    (status, x kv buffer, G); status 2 when G >= 1.  E (kv, n x n) replaces
    the product R [A] when given."""
    x = np.zeros(2 * n * nrhs)
    g = np.zeros(1)
    st = lib().orc_ilss_verify(n, nrhs, _p(A), _p(b), _p(R), _p(mx),
                               None if E is None else _p(E), _p(x), _p(g), int(threads))
    return int(st), x, float(g[0])


def ref_imats_linearsolve(n, nrhs, A, b):
    """The reference's imats<double, pidblas>::linearsolve run as is:
    (status, x, R, mx) with R, mx the approximate inverse and solution it
    used; None where the reference build is absent."""
    Rl = ref_lib()
    if Rl is None:
        return None
    x = np.zeros(2 * n * nrhs)
    R = np.zeros(n * n)
    mx = np.zeros(n * nrhs)
    st = Rl.ref_imats_linearsolve(n, nrhs, _p(A), _p(b), _p(x), _p(R), _p(mx))
    return int(st), x, R, mx


def ieigsymge(n, A, B, X, lam, Y, C=None, BX=None, R=None, S=None, merge=True, threads=0):
    """imats::eigsymge's verification (restatement) for given X, lambda, Y:
    (status, enclosures kv (n), bound ||YBX - I||); status 2 when the bound
    is >= 1.  C, BX, R, S replace the products [A]X, [B]X, YC, Y[BX]."""
    out = np.zeros(2 * n)
    g = np.zeros(1)
    opt = [None if v is None else _p(v) for v in (C, BX, R, S)]
    st = lib().orc_ieigsymge(n, _p(A), _p(B), _p(X), _p(lam), _p(Y), *opt, _p(out), _p(g),
                             int(merge), int(threads))
    return int(st), out, float(g[0])


def imats_mul_m_im_naive(m, n, k, Y, C):
    """imats::mul_m_im 'M' x 'M' (restatement): Y point (m x k) times C kv."""
    R = np.zeros(2 * m * n)
    lib().orc_imats_mul_m_im_naive(m, n, k, _p(Y), _p(C), _p(R))
    return R


def ref_imats_eigsymge(n, A, B):
    """The reference's imats<double, pidblas>::eigsymge run as is:
    (status, enclosures kv (n), X, lambda, Y); None without the reference."""
    Rl = ref_lib()
    if Rl is None:
        return None
    lam = np.zeros(2 * n)
    X = np.zeros(n * n)
    lmb = np.zeros(n)
    Y = np.zeros(n * n)
    st = Rl.ref_imats_eigsymge(n, _p(A), _p(B), _p(lam), _p(X), _p(lmb), _p(Y))
    return int(st), lam, X, lmb, Y


def ifma(A, B, C_) -> np.ndarray:
    """vcp::ifma elementwise over kv buffers (restatement)."""
    n = A.size // 2
    R = np.empty(2 * n)
    lib().orc_ifma(n, _p(A), _p(B), _p(C_), _p(R))
    return R


def pidblas_fma_mulmm(m, n, k, A, B, threads=0) -> np.ndarray:
    """vcp::pidblas_fma::mulmm (restatement), kv buffers, GEMM naming."""
    C_ = np.empty(2 * m * n)
    lib().orc_pidblas_fma_mulmm(m, n, k, _p(A), _p(B), _p(C_), int(threads))
    return C_


def tensor_basis(nb, ia, ib, nt, Ta, Tb, nqa, nqb, out, ld, s1=None, s2=None,
                 transposed=False, accumulate=False, offset=0, threads=0):
    """The tensor-product basis matrix of the GPU's vcpcu_tensor_basis_dev
    (restatement, same roundings): writes into the kv buffer out from
    double offset `offset`."""
    ia = np.ascontiguousarray(ia, dtype=np.int32)
    ib = np.ascontiguousarray(ib, dtype=np.int32)
    o = out[offset:]
    lib().orc_tensor_basis(int(nb), _p(ia), _p(ib), int(nt), _p(Ta), _p(Tb), int(nqa), int(nqb),
                           None if s1 is None else _p(s1), None if s2 is None else _p(s2),
                           _p(o), C.c_long(int(ld)), int(transposed), int(accumulate),
                           int(threads))
    return out


def pddblas_mulmm(m, n, k, A, B, threads=0) -> np.ndarray:
    """pddblas::mulmm (restatement): dd kv pairs, GEMM naming."""
    C_ = np.empty(2 * m * n)
    lib().orc_pddblas_mulmm(m, n, k, _p(A), _p(B), _p(C_), int(threads))
    return C_


def pddblas_mulltmm(m, nc, A, threads=0) -> np.ndarray:
    """pddblas::mulltmm (restatement): A^T A for a dd A (m x nc)."""
    C_ = np.empty(2 * nc * nc)
    lib().orc_pddblas_mulltmm(m, nc, _p(A), _p(C_), int(threads))
    return C_


def fp64_peak_gflops(seconds=0.5, threads=0) -> float:
    """Measured FP64 FMA throughput of the host cores (GFLOP/s)."""
    return float(lib().orc_fp64_peak(float(seconds), int(threads)))


def ref_pddblas_mulmm(m, n, k, A, B):
    """The reference's pddblas::mulmm as built here; None without it."""
    R = ref_lib()
    if R is None:
        return None
    C_ = np.empty(2 * m * n)
    assert R.ref_pddblas_mulmm(m, n, k, _p(A), _p(B), _p(C_)) == 0
    return C_


def ref_pddblas_mulltmm(m, nc, A):
    R = ref_lib()
    if R is None:
        return None
    C_ = np.empty(2 * nc * nc)
    assert R.ref_pddblas_mulltmm(m, nc, _p(A), _p(C_)) == 0
    return C_


def ref_call(name, *args):
    """Call a reference-build wrapper; None where the reference is absent."""
    R = ref_lib()
    if R is None:
        return None
    return getattr(R, name)(*args)


def exact_sum(x: np.ndarray, direction: int) -> float:
    x = np.ascontiguousarray(x, dtype=np.float64)
    return float(lib().orc_exact_sum(x.size, _p(x), int(direction)))


def ref_rmatmul(m, n, k, A, B, rnd) -> np.ndarray | None:
    R = ref_lib()
    if R is None:
        return None
    C_ = np.zeros(max(m * k, 1), dtype=np.float64)
    R.ref_rmatmul(m, n, k, _p(A), _p(B), _p(C_), int(rnd))
    return C_


def ref_pidblas_mulmm(m, n, k, A, B) -> np.ndarray | None:
    R = ref_lib()
    if R is None:
        return None
    C_ = np.zeros(2 * m * n, dtype=np.float64)
    st = R.ref_pidblas_mulmm(m, n, k, _p(A), _p(B), _p(C_))
    assert st == 0
    return C_
