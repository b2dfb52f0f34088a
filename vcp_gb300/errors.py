"""Exceptions raised for non-zero C ABI statuses.

They mirror the vcp::error hierarchy (vcp/error.hpp): a bad shape becomes a
DimensionError (vcp::dimension_error), an unusable state a StateError
(vcp::state_error) and a failed verification a VerificationError
(vcp::verification_error, vcp/error.hpp:77).
"""
from __future__ import annotations

OK = 0
ERR_INVALID_ARG = 1
ERR_CUDA = 2
ERR_NONFINITE = 3
ERR_RANGE = 4
ERR_TIMEOUT = 5
ERR_UNSUPPORTED = 6
ERR_ALLOC = 7
ERR_VERIFY = 8
ERR_IO = 9


class VcpError(RuntimeError):
    status = -1


class DimensionError(VcpError):
    status = ERR_INVALID_ARG


class StateError(VcpError):
    pass


class VerificationError(VcpError):
    status = ERR_VERIFY


class CudaError(StateError):
    status = ERR_CUDA


class NonFiniteError(StateError):
    status = ERR_NONFINITE


class RangeError(StateError):
    status = ERR_RANGE


class TimeoutError_(StateError):
    status = ERR_TIMEOUT


class UnsupportedError(StateError):
    status = ERR_UNSUPPORTED


class AllocError(StateError):
    status = ERR_ALLOC


class IOError_(VcpError):
    """vcp::io_error (vcp/error.hpp): a .vcpmat file could not be read or written."""
    status = ERR_IO


_BY_STATUS = {c.status: c for c in (DimensionError, CudaError, NonFiniteError, RangeError,
                                     TimeoutError_, UnsupportedError, AllocError,
                                     VerificationError, IOError_)}


def raise_for_status(status: int, msg: str) -> None:
    if status == OK:
        return
    raise _BY_STATUS.get(status, VcpError)(f"[status {status}] {msg}")
