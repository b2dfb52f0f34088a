"""Interval GEMM with pidblas semantics on the GPU (the ``vcp::pidcuda`` policy).

Interval matrices use the kv::interval<double> memory layout: column-major,
each entry a pair {inf, sup} of doubles.  As numpy arrays they are float64
buffers of 2*rows*cols doubles; ``to_kv`` / ``from_kv`` convert from / to a
pair of (rows x cols) endpoint arrays.

``mulmm(A, B, m, n, k, form)`` computes C = A * B for A (m x k) and B (k x n)
the way pidblas::mulmm does (vcp/pidblas.hpp:239-294): midpoint-radius form,
lower end RD(mA*mB) - T, upper end RU(mA*mB) + T with
T = RU((|mA|+rA)*rB + rA*|mB|).  ``form`` selects the plain FP64 kernels
(bit-identical to pidblas over a sequential-chain dgemm) or the Ozaki form
on the tensor cores.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .vblas import _dev_ptr, _host_ptr, _stream_ptr

FORM_PLAIN = 0
FORM_OZAKI = 1
FORM_AUTO = 2
FORM_OZAKI_SLICES = 3
# added to `slices` of FORM_OZAKI: radius products without their low x low
# digit pair, bounded instead (VCPCU_SLICES_FAST_RADIUS)
SLICES_FAST_RADIUS = 0x100


def to_kv(lo: np.ndarray, up: np.ndarray) -> np.ndarray:
    """(rows x cols) endpoint arrays -> flat kv-layout buffer (column-major)."""
    lo = np.asarray(lo, dtype=np.float64)
    up = np.asarray(up, dtype=np.float64)
    if lo.shape != up.shape or lo.ndim != 2:
        raise ValueError("lo and up must be 2-D arrays of one shape")
    out = np.empty((lo.shape[1], lo.shape[0], 2), dtype=np.float64)
    out[:, :, 0] = lo.T
    out[:, :, 1] = up.T
    return out.reshape(-1)


def from_kv(buf: np.ndarray, rows: int, cols: int) -> tuple[np.ndarray, np.ndarray]:
    """Flat kv-layout buffer -> (lo, up), each (rows x cols)."""
    v = np.asarray(buf).reshape(cols, rows, 2)
    return v[:, :, 0].T.copy(), v[:, :, 1].T.copy()


def mulmm(A: np.ndarray, B: np.ndarray, m: int, n: int, k: int, form: int = FORM_PLAIN,
          slices: int = 0, out: np.ndarray | None = None) -> np.ndarray:
    """Host-pointer interval product (synchronous).  Returns the kv buffer of C."""
    if out is None:
        out = np.empty(2 * m * n, dtype=np.float64)
    if m <= 0 or n <= 0:
        return out
    pa = _host_ptr(A, 2 * m * k, "A") if k > 0 else None
    pb = _host_ptr(B, 2 * k * n, "B") if k > 0 else None
    pc = _host_ptr(out, 2 * m * n, "C", writable=True)
    _lib.call("vcpcu_igemm", m, n, k, pa, pb, pc, int(form), int(slices))
    return out


def mulmm_dev(m, n, k, A, lda, B, ldb, C, ldc, form=FORM_PLAIN, slices=0, stream=None) -> None:
    """Device-pointer interval product on a CUDA stream (torch tensors)."""
    _lib.call("vcpcu_igemm_dev", m, n, k, _dev_ptr(A, "A"), lda, _dev_ptr(B, "B"), ldb,
              _dev_ptr(C, "C"), ldc, int(form), int(slices), _stream_ptr(stream))


# ---- interval x point, [A]^T[A], verified A^T A, ||R[A] - I|| ------------------

def mul_point(interval_side: int, L: np.ndarray, R: np.ndarray, m: int, n: int, k: int,
              form: int = FORM_PLAIN, slices: int = 0) -> np.ndarray:
    """interval_side 0: [L] * R (pidblas::mul_im_m); 1: L * [R] (pidblas::mul_m_im).
    The interval factor is a kv buffer, the point factor a float64 buffer."""
    out = np.empty(2 * m * n, dtype=np.float64)
    if m <= 0 or n <= 0:
        return out
    wl, wr = (2, 1) if interval_side == 0 else (1, 2)
    pl = _host_ptr(L, wl * m * k, "L") if k > 0 else None
    pr = _host_ptr(R, wr * k * n, "R") if k > 0 else None
    _lib.call("vcpcu_igemm_point", int(interval_side), m, n, k, pl, pr, out.ctypes.data,
              int(form), int(slices))
    return out


def isyrk(A: np.ndarray, n: int, k: int, form: int = FORM_PLAIN, slices: int = 0) -> np.ndarray:
    """[A]^T [A] for an interval A (k x n): pidblas::mulltmm."""
    out = np.empty(2 * n * n, dtype=np.float64)
    if n <= 0:
        return out
    pa = _host_ptr(A, 2 * k * n, "A") if k > 0 else None
    _lib.call("vcpcu_isyrk", n, k, pa, out.ctypes.data, int(form), int(slices))
    return out


def vsyrk(A: np.ndarray, n: int, k: int) -> np.ndarray:
    """Verified A^T A of a point A (k x n): pidblas::vmulmm."""
    out = np.empty(2 * n * n, dtype=np.float64)
    if n <= 0:
        return out
    pa = _host_ptr(A, k * n, "A") if k > 0 else None
    _lib.call("vcpcu_vsyrk", n, k, pa, out.ctypes.data)
    return out


def norm_I_minus_RA(R: np.ndarray, A: np.ndarray, n: int, form: int = FORM_PLAIN,
                    slices: int = 0) -> float:
    """Upper bound of ||R [A] - I||_inf (the check of imats::linearsolve)."""
    import ctypes
    out = ctypes.c_double(0.0)
    _lib.call("vcpcu_norm_I_minus_RA", n, _host_ptr(R, n * n, "R"), _host_ptr(A, 2 * n * n, "A"),
              ctypes.addressof(out), int(form), int(slices))
    return out.value


def linearsolve_verify(A: np.ndarray, b: np.ndarray, R: np.ndarray, mx: np.ndarray, n: int,
                       nrhs: int, form: int = FORM_PLAIN, slices: int = 0,
                       check: bool = True) -> tuple[np.ndarray, float]:
    """The verification of imats::linearsolve (vcp/imats.hpp:293-364) for the
    approximate inverse R of mid(A) and the approximate solution mx = R mid(b):
    returns (x, G) with x the kv buffer of the enclosure (n x nrhs) and G the
    upper bound of ||RA - I||_inf.  With check, G >= 1 raises
    VerificationError as the reference throws vcp::verification_error."""
    import ctypes
    x = np.empty(2 * n * nrhs, dtype=np.float64)
    g = ctypes.c_double(0.0)
    lib = _lib.load()
    st = lib.vcpcu_ilss_verify(n, nrhs, _host_ptr(A, 2 * n * n, "A"),
                               _host_ptr(b, 2 * n * nrhs, "b"), _host_ptr(R, n * n, "R"),
                               _host_ptr(mx, n * nrhs, "mx"), x.ctypes.data, ctypes.addressof(g),
                               int(form), int(slices))
    if st != 0 and (check or st != 8):
        from .errors import raise_for_status
        raise_for_status(st, "vcpcu_ilss_verify: " +
                         lib.vcpcu_last_error_string().decode(errors="replace"))
    return x, g.value


def linearsolve_verify_dev(n, nrhs, A, lda, b, ldb, R, ldr, mx, ldmx, x, ldx, bound,
                           form=FORM_PLAIN, slices=0, stream=None) -> None:
    """Device-pointer form on a CUDA stream; bound (one double) stays on the
    device, the caller tests bound < 1."""
    _lib.call("vcpcu_ilss_verify_dev", n, nrhs, _dev_ptr(A, "A"), lda, _dev_ptr(b, "b"), ldb,
              _dev_ptr(R, "R"), ldr, _dev_ptr(mx, "mx"), ldmx, _dev_ptr(x, "x"), ldx,
              _dev_ptr(bound, "bound"), int(form), int(slices), _stream_ptr(stream))


_INVERSE_FN = None


def _inverse_fn_type():
    global _INVERSE_FN
    if _INVERSE_FN is None:
        import ctypes
        _INVERSE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_void_p)
    return _INVERSE_FN


def eigsymge_verify(A: np.ndarray, B: np.ndarray, X: np.ndarray, lam: np.ndarray, n: int,
                    inverse=None, form: int = FORM_PLAIN, slices: int = 0,
                    check: bool = True) -> tuple[np.ndarray, float]:
    """The verification of imats::eigsymge (vcp/imats.hpp:419-522) around the
    approximate eigenvectors X (n x n, column-major) and eigenvalues lam of
    mid(A) x = lam mid(B) x: returns (kv buffer of the n merged eigenvalue
    enclosures, sup ||Y B X - I||).  ``inverse(M)`` turns mid(B X) (n x n
    numpy array) into Y ~ inv(mid(B X)) (default numpy.linalg.inv).  With
    check, a bound >= 1 raises VerificationError as the reference throws."""
    import ctypes
    inv = np.linalg.inv if inverse is None else inverse

    def cb(nn, ptr, _ctx):
        try:
            M = np.ctypeslib.as_array(ptr, shape=(nn * nn,))
            Y = np.asarray(inv(M.reshape(nn, nn, order="F").copy()), dtype=np.float64)
            M[:] = Y.ravel(order="F")
            return 0
        except Exception:
            return 1

    fn = _inverse_fn_type()(cb)
    out = np.empty(2 * n, dtype=np.float64)
    g = ctypes.c_double(0.0)
    lib = _lib.load()
    st = lib.vcpcu_ieigsymge(n, _host_ptr(A, 2 * n * n, "A"), _host_ptr(B, 2 * n * n, "B"),
                             _host_ptr(X, n * n, "X"), _host_ptr(lam, n, "lambda"),
                             ctypes.cast(fn, ctypes.c_void_p), None, out.ctypes.data,
                             ctypes.addressof(g), int(form), int(slices))
    if st != 0 and (check or st != 8):
        from .errors import raise_for_status
        raise_for_status(st, "vcpcu_ieigsymge: " +
                         lib.vcpcu_last_error_string().decode(errors="replace"))
    return out, g.value


def eigsymge_stage1_dev(n, A, lda, B, ldb, X, ldx, C, BX, midBX, form=FORM_PLAIN, slices=0,
                        stream=None) -> None:
    _lib.call("vcpcu_ieigsymge_stage1_dev", n, _dev_ptr(A, "A"), lda, _dev_ptr(B, "B"), ldb,
              _dev_ptr(X, "X"), ldx, _dev_ptr(C, "C"), _dev_ptr(BX, "BX"),
              _dev_ptr(midBX, "midBX"), int(form), int(slices), _stream_ptr(stream))


def eigsymge_stage2_dev(n, lam, Y, ldy, C, BX, out, bound, form=FORM_PLAIN, slices=0,
                        stream=None) -> None:
    _lib.call("vcpcu_ieigsymge_stage2_dev", n, _dev_ptr(lam, "lambda"), _dev_ptr(Y, "Y"), ldy,
              _dev_ptr(C, "C"), _dev_ptr(BX, "BX"), _dev_ptr(out, "lam"),
              _dev_ptr(bound, "bound"), int(form), int(slices), _stream_ptr(stream))


def eig_merge(lam_kv: np.ndarray, n: int) -> np.ndarray:
    """The overlap merge of imats::eigsymge, in place on a kv buffer of n."""
    _lib.call("vcpcu_eig_merge", n, _host_ptr(lam_kv, 2 * n, "lam", writable=True))
    return lam_kv


# ---- AUTO form -------------------------------------------------------------------

def autotune(stream=None) -> dict:
    """Measure the cost-model constants of FORM_AUTO on the current GPU (one
    plain and two Ozaki products) and keep them for the process; stored in
    the file named by VCPCU_AUTOTUNE_CACHE when that variable is set."""
    c = np.zeros(4, dtype=np.float64)
    _lib.call("vcpcu_autotune", _stream_ptr(stream), c.ctypes.data)
    return dict(fp64_rate=c[0], tc_rate=c[1], prep_bw=c[2], t_launch=c[3])


def autotune_choice(m: int, n: int, k: int, batched: bool = False) -> int:
    """The form (FORM_PLAIN or FORM_OZAKI) that FORM_AUTO uses for m x n x k,
    as a single product or as one problem of a batch."""
    return int(_lib.load().vcpcu_autotune_choice(int(m), int(n), int(k), int(bool(batched))))


def autotune_pick(A, B, m: int, n: int, k: int, stream=None) -> tuple[int, int]:
    """(form, slices) that FORM_AUTO uses for [A] [B] (kv buffers: numpy
    host arrays or float64 CUDA tensors): the tensor-core slice count whose
    enclosures are no wider than the plain form's on a probe (possibly with
    SLICES_FAST_RADIUS added), or FORM_PLAIN."""
    import ctypes
    f, s = ctypes.c_int(0), ctypes.c_int(0)
    if isinstance(A, np.ndarray):
        pa, pb = _host_ptr(A, 2 * m * k, "A"), _host_ptr(B, 2 * k * n, "B")
    else:
        pa, pb = _dev_ptr(A, "A"), _dev_ptr(B, "B")
    _lib.call("vcpcu_autotune_pick", m, n, k, pa, m, pb, k, ctypes.addressof(f),
              ctypes.addressof(s), _stream_ptr(stream))
    return f.value, s.value


# ---- inf-sup interval FMA (vcp::ifma) and its product (vcp::pidblas_fma) ------------

def ifma(A: np.ndarray, B: np.ndarray, C: np.ndarray) -> np.ndarray:
    """Elementwise vcp::ifma over kv buffers: R = [A] [B] + [C] (inf-sup form,
    directed fused multiply-adds; vcp/ifma.hpp:48-139)."""
    n = np.asarray(A).size // 2
    R = np.empty(2 * n, dtype=np.float64)
    if n == 0:
        return R
    _lib.call("vcpcu_ifma", n, _host_ptr(A, 2 * n, "A"), _host_ptr(B, 2 * n, "B"),
              _host_ptr(C, 2 * n, "C"), _host_ptr(R, 2 * n, "R", writable=True))
    return R


def mulmm_fma(A: np.ndarray, B: np.ndarray, m: int, n: int, k: int) -> np.ndarray:
    """C = [A] [B] as vcp::pidblas_fma::mulmm (an ifma chain per entry, ascending
    inner index; vcp/pidblas_fma.hpp:46-80).  Returns the kv buffer of C."""
    out = np.empty(2 * m * n, dtype=np.float64)
    if m <= 0 or n <= 0:
        return out
    pa = _host_ptr(A, 2 * m * k, "A") if k > 0 else None
    pb = _host_ptr(B, 2 * k * n, "B") if k > 0 else None
    _lib.call("vcpcu_igemm_fma", m, n, k, pa, pb, _host_ptr(out, 2 * m * n, "C", writable=True))
    return out


def mulmm_fma_dev(m, n, k, A, lda, B, ldb, C, ldc, stream=None) -> None:
    _lib.call("vcpcu_igemm_fma_dev", m, n, k, _dev_ptr(A, "A"), lda, _dev_ptr(B, "B"), ldb,
              _dev_ptr(C, "C"), ldc, _stream_ptr(stream))
