"""Portable matrix files (.vcpmat, the format of vcp::save_portable /
load_portable, vcp/vcp_portable_fio.hpp) through libvcpcuda.

Arrays are column-major element buffers in the kv layouts: int32 and double
as is, ``interval`` / ``dd`` as 2 doubles per element ({lower, upper} /
{a1, a2}), ``interval_dd`` as 4 ({lo.a1, lo.a2, up.a1, up.a2}).  ``name`` is
the file name without the ``.vcpmat`` suffix, as in the reference.

    vcpmat.save("A", kv_buffer, rows, cols, "interval")
    buf, kind, rows, cols = vcpmat.load("A")
    vcpmat.load_dev("A", tensor, ld, stream)      # straight into device memory
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .vblas import _dev_ptr, _stream_ptr

KINDS = {"int32": 1, "double": 2, "interval": 3, "dd": 4, "interval_dd": 5}
_NAMES = {v: k for k, v in KINDS.items()}
_WIDTH = {1: 1, 2: 1, 3: 2, 4: 2, 5: 4}  # array items per element


def _kind(kind) -> int:
    return KINDS[kind] if isinstance(kind, str) else int(kind)


def info(name: str) -> tuple[str, int, int]:
    """(kind, rows, cols) from the file's header (checked)."""
    t, r, c = C.c_int(0), C.c_int(0), C.c_int(0)
    _lib.call("vcpcu_vcpmat_info", name.encode(), C.byref(t), C.byref(r), C.byref(c))
    return _NAMES[t.value], r.value, c.value


def save(name: str, data: np.ndarray, rows: int, cols: int, kind="double") -> None:
    t = _kind(kind)
    dtype = np.int32 if t == 1 else np.float64
    a = np.ascontiguousarray(data, dtype=dtype)
    if a.size != rows * cols * _WIDTH[t]:
        raise ValueError(f"{a.size} items for a {rows} x {cols} matrix of kind {_NAMES[t]}")
    _lib.call("vcpcu_vcpmat_save", name.encode(), t, rows, cols, a.ctypes.data if a.size else None)


def load(name: str, kind=None) -> tuple[np.ndarray, str, int, int]:
    """(buffer, kind, rows, cols); with ``kind`` the file must hold that type."""
    k, rows, cols = info(name)
    t = KINDS[k] if kind is None else _kind(kind)
    out = np.empty(rows * cols * _WIDTH[t], dtype=np.int32 if t == 1 else np.float64)
    _lib.call("vcpcu_vcpmat_load", name.encode(), t, rows, cols,
              out.ctypes.data if out.size else None)
    return out, _NAMES[t], rows, cols


def save_dev(name: str, tensor, rows: int, cols: int, ld: int, kind="interval",
             stream=None) -> None:
    """Write a device matrix (torch tensor, leading dimension ``ld`` in elements)."""
    _lib.call("vcpcu_vcpmat_save_dev", name.encode(), _kind(kind), rows, cols,
              _dev_ptr(tensor, "data") if rows else None, ld, _stream_ptr(stream))


def load_dev(name: str, tensor, ld: int, kind=None, stream=None) -> tuple[str, int, int]:
    """Read a file into a device matrix (leading dimension ``ld`` in elements)."""
    k, rows, cols = info(name)
    t = KINDS[k] if kind is None else _kind(kind)
    _lib.call("vcpcu_vcpmat_load_dev", name.encode(), t, rows, cols,
              _dev_ptr(tensor, "data") if rows else None, ld, _stream_ptr(stream))
    return _NAMES[t], rows, cols
