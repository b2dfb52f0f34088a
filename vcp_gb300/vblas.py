"""Directed-rounding point GEMM with the vblas signatures, on the GPU.

``rmatmul(m, n, k, A, B, C, rounding_mode)`` mirrors vblas ``rmatmul``
(vblas/rmatmul.hpp:102) argument for argument: A is m x n, B is n x k and C is
m x k, all column-major (pass flat float64 buffers, or Fortran-ordered 2-D
arrays); C is overwritten; rounding_mode is 1 (up), -1 (down) or anything
else (nearest).  ``udmatmul`` mirrors vblas/udmatmul.hpp:758.  Each result
entry is the ascending sequential FMA chain of the inner index, rounded per
instruction on the GPU, so results are bit-identical to vblas.

The ``*_dev`` forms take CUDA tensors (torch) and leading dimensions, and are
ordered on the given CUDA stream (default: torch's current stream).
"""
from __future__ import annotations

import numpy as np

from . import _lib


def _host_ptr(a: np.ndarray, need: int, name: str, writable: bool = False) -> int:
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise TypeError(f"{name} must be a float64 numpy array")
    if need and a.size < need:
        raise ValueError(f"{name} holds {a.size} doubles, needs {need}")
    if not (a.flags.f_contiguous or a.flags.c_contiguous):
        raise ValueError(f"{name} must be contiguous")
    if writable and not a.flags.writeable:
        raise ValueError(f"{name} must be writable")
    return a.ctypes.data


def rmatmul(m: int, n: int, k: int, A: np.ndarray, B: np.ndarray, C: np.ndarray,
            rounding_mode: int) -> None:
    if m <= 0 or k <= 0:
        return
    pa = _host_ptr(A, m * n, "A") if n > 0 else None
    pb = _host_ptr(B, n * k, "B") if n > 0 else None
    pc = _host_ptr(C, m * k, "C", writable=True)
    _lib.call("vcpcu_rmatmul", m, n, k, pa, pb, pc, int(rounding_mode))


def udmatmul(m: int, n: int, k: int, A: np.ndarray, B: np.ndarray, CU: np.ndarray,
             CD: np.ndarray) -> None:
    if m <= 0 or k <= 0:
        return
    pa = _host_ptr(A, m * n, "A") if n > 0 else None
    pb = _host_ptr(B, n * k, "B") if n > 0 else None
    pu = _host_ptr(CU, m * k, "CU", writable=True)
    pd = _host_ptr(CD, m * k, "CD", writable=True)
    _lib.call("vcpcu_udmatmul", m, n, k, pa, pb, pu, pd)


def _stream_ptr(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _dev_ptr(t, name: str) -> int:
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64:
        raise TypeError(f"{name} must be a float64 CUDA tensor")
    return t.data_ptr()


def rmatmul_dev(m, n, k, A, lda, B, ldb, C, ldc, rounding_mode, stream=None) -> None:
    _lib.call("vcpcu_rmatmul_dev", m, n, k, _dev_ptr(A, "A"), lda, _dev_ptr(B, "B"), ldb,
              _dev_ptr(C, "C"), ldc, int(rounding_mode), _stream_ptr(stream))


def udmatmul_dev(m, n, k, A, lda, B, ldb, CU, CD, ldc, stream=None) -> None:
    _lib.call("vcpcu_udmatmul_dev", m, n, k, _dev_ptr(A, "A"), lda, _dev_ptr(B, "B"), ldb,
              _dev_ptr(CU, "CU"), _dev_ptr(CD, "CD"), ldc, _stream_ptr(stream))


def udmatmul_ozaki(m: int, n: int, k: int, A: np.ndarray, B: np.ndarray, CU: np.ndarray,
                   CD: np.ndarray, slices: int = 0) -> None:
    """CD <= A B <= CU on the tensor cores (Ozaki form; not the FMA-chain bits)."""
    if m <= 0 or k <= 0:
        return
    pa = _host_ptr(A, m * n, "A") if n > 0 else None
    pb = _host_ptr(B, n * k, "B") if n > 0 else None
    pu = _host_ptr(CU, m * k, "CU", writable=True)
    pd = _host_ptr(CD, m * k, "CD", writable=True)
    _lib.call("vcpcu_udmatmul_ozaki", m, n, k, pa, pb, pu, pd, int(slices))


def udmatmul_ozaki_dev(m, n, k, A, lda, B, ldb, CU, CD, ldc, slices=0, stream=None) -> None:
    _lib.call("vcpcu_udmatmul_ozaki_dev", m, n, k, _dev_ptr(A, "A"), lda, _dev_ptr(B, "B"), ldb,
              _dev_ptr(CU, "CU"), _dev_ptr(CD, "CD"), ldc, int(slices), _stream_ptr(stream))
