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
