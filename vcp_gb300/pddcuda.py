"""Double-double GEMM with pddblas semantics on the GPU (the vcp::pddcuda policy).

dd matrices use the kv::dd memory layout: column-major, each entry a pair
{a1, a2} of doubles (value a1 + a2).  ``mulmm(A, B, m, n, k)`` returns the dd
product C (kv buffer) and a rigorous per-entry upper bound of |AB - C|
(vcp/pddblas.hpp:318-376 computes the same product, approximately, with
double slices and dd accumulation).
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .vblas import _dev_ptr, _host_ptr, _stream_ptr


def mulmm(A: np.ndarray, B: np.ndarray, m: int, n: int, k: int, slices: int = 0,
          with_bound: bool = True):
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
