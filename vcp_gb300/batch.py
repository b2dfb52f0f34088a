"""Batches of uneven interval GEMMs (vcpcu_igemm_batched_dev, vcpcu_batch_graph_*).

A problem is (m, n, k, A, lda, B, ldb, C, ldc) with A, B, C device buffers
(torch float64 CUDA tensors) in kv interval layout.  ``run`` executes a batch
once; ``BatchGraph`` captures it into a CUDA graph and replays it with one
launch, reporting per-problem latencies from device clock stamps.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .vblas import _dev_ptr, _stream_ptr


class Problem(C.Structure):
    _fields_ = [("m", C.c_int), ("n", C.c_int), ("k", C.c_int), ("lda", C.c_int),
                ("ldb", C.c_int), ("ldc", C.c_int), ("A", C.c_void_p), ("B", C.c_void_p),
                ("C", C.c_void_p)]


def table(problems) -> C.Array:
    """problems: iterable of (m, n, k, A, lda, B, ldb, Cout, ldc) with CUDA tensors."""
    rows = []
    for (m, n, k, A, lda, B, ldb, Cc, ldc) in problems:
        rows.append(Problem(m, n, k, lda, ldb, ldc, _dev_ptr(A, "A"), _dev_ptr(B, "B"),
                            _dev_ptr(Cc, "C")))
    arr = (Problem * len(rows))(*rows)
    return arr


def run(problems, form: int, slices: int = 0, stream=None) -> None:
    t = table(problems)
    _lib.call("vcpcu_igemm_batched_dev", len(t), C.cast(t, C.c_void_p), int(form), int(slices),
              _stream_ptr(stream))


class BatchGraph:
    def __init__(self, problems, form: int, slices: int = 0, stream=None):
        self._t = table(problems)
        self.count = len(self._t)
        self._h = C.c_void_p(0)
        _lib.call("vcpcu_batch_graph_create", self.count, C.cast(self._t, C.c_void_p), int(form),
                  int(slices), _stream_ptr(stream), C.byref(self._h))

    def launch(self, stream=None) -> None:
        _lib.call("vcpcu_batch_graph_launch", self._h, _stream_ptr(stream))

    def latencies(self, stream=None) -> tuple[np.ndarray, np.ndarray]:
        """(start_us, latency_us) per problem of the last replay (synchronises)."""
        st = np.zeros(self.count)
        la = np.zeros(self.count)
        _lib.call("vcpcu_batch_graph_latencies", self._h, _stream_ptr(stream), st.ctypes.data,
                  la.ctypes.data)
        return st, la

    def close(self) -> None:
        if self._h:
            _lib.call("vcpcu_batch_graph_destroy", self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
