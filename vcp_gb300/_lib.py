"""ctypes binding of libvcpcuda.so (the C ABI declared in include/vcpcuda.h).

There is no fallback: if the shared library is missing or cannot be loaded,
every entry point raises.  Build it with ``vcp_gb300.build.build()``.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from .errors import raise_for_status

LIB_PATH = Path(__file__).resolve().parent / "libvcpcuda.so"

_lock = threading.Lock()
_lib: C.CDLL | None = None

_i, _d, _v, _ll = C.c_int, C.POINTER(C.c_double), C.c_void_p, C.c_longlong

# name -> (restype, argtypes); must match include/vcpcuda.h
SIGNATURES: dict[str, tuple] = {
    "vcpcu_last_error_string": (C.c_char_p, []),
    "vcpcu_version": (_i, []),
    "vcpcu_launch_count": (_ll, []),
    "vcpcu_status": (_i, [_v]),
    "vcpcu_profile": (_i, [_i]),
    "vcpcu_profile_read": (_i, [_v, _i, _v]),
    "vcpcu_rmatmul": (_i, [_i, _i, _i, _v, _v, _v, _i]),
    "vcpcu_udmatmul": (_i, [_i, _i, _i, _v, _v, _v, _v]),
    "vcpcu_rmatmul_dev": (_i, [_i, _i, _i, _v, _i, _v, _i, _v, _i, _i, _v]),
    "vcpcu_udmatmul_dev": (_i, [_i, _i, _i, _v, _i, _v, _i, _v, _v, _i, _v]),
    "vcpcu_igemm_dev": (_i, [_i, _i, _i, _v, _i, _v, _i, _v, _i, _i, _i, _v]),
    "vcpcu_igemm": (_i, [_i, _i, _i, _v, _v, _v, _i, _i]),
    "vcpcu_igemm_point_dev": (_i, [_i, _i, _i, _i, _v, _i, _v, _i, _v, _i, _i, _i, _v]),
    "vcpcu_igemm_point": (_i, [_i, _i, _i, _i, _v, _v, _v, _i, _i]),
    "vcpcu_isyrk_dev": (_i, [_i, _i, _v, _i, _v, _i, _i, _i, _v]),
    "vcpcu_isyrk": (_i, [_i, _i, _v, _v, _i, _i]),
    "vcpcu_vsyrk_dev": (_i, [_i, _i, _v, _i, _v, _i, _v]),
    "vcpcu_vsyrk": (_i, [_i, _i, _v, _v]),
    "vcpcu_norm_I_minus_RA_dev": (_i, [_i, _v, _i, _v, _i, _v, _i, _i, _v]),
    "vcpcu_norm_I_minus_RA": (_i, [_i, _v, _v, _v, _i, _i]),
    "vcpcu_ilss_verify_dev": (_i, [_i, _i, _v, _i, _v, _i, _v, _i, _v, _i, _v, _i, _v, _i, _i,
                                   _v]),
    "vcpcu_ilss_verify": (_i, [_i, _i, _v, _v, _v, _v, _v, _v, _i, _i]),
    "vcpcu_ieigsymge_stage1_dev": (_i, [_i, _v, _i, _v, _i, _v, _i, _v, _v, _v, _i, _i, _v]),
    "vcpcu_ieigsymge_stage2_dev": (_i, [_i, _v, _v, _i, _v, _v, _v, _v, _i, _i, _v]),
    "vcpcu_eig_merge": (_i, [_i, _v]),
    "vcpcu_selftest_timeout": (_i, [C.c_longlong, _v]),
    "vcpcu_ieigsymge": (_i, [_i, _v, _v, _v, _v, _v, _v, _v, _v, _i, _i]),
    "vcpcu_vcpmat_save": (_i, [C.c_char_p, _i, _i, _i, _v]),
    "vcpcu_vcpmat_info": (_i, [C.c_char_p, _v, _v, _v]),
    "vcpcu_vcpmat_load": (_i, [C.c_char_p, _i, _i, _i, _v]),
    "vcpcu_vcpmat_save_dev": (_i, [C.c_char_p, _i, _i, _i, _v, _i, _v]),
    "vcpcu_vcpmat_load_dev": (_i, [C.c_char_p, _i, _i, _i, _v, _i, _v]),
    "vcpcu_ddgemm_dev": (_i, [_i, _i, _i, _v, _i, _v, _i, _v, _i, _v, _i, _i, _v]),
    "vcpcu_ddgemm": (_i, [_i, _i, _i, _v, _v, _v, _v, _i]),
    "vcpcu_udmatmul_ozaki_dev": (_i, [_i, _i, _i, _v, _i, _v, _i, _v, _v, _i, _i, _v]),
    "vcpcu_udmatmul_ozaki": (_i, [_i, _i, _i, _v, _v, _v, _v, _i]),
    "vcpcu_ifma_dev": (_i, [C.c_long, _v, _v, _v, _v, _v]),
    "vcpcu_ifma": (_i, [C.c_long, _v, _v, _v, _v]),
    "vcpcu_igemm_fma_dev": (_i, [_i, _i, _i, _v, _i, _v, _i, _v, _i, _v]),
    "vcpcu_igemm_fma": (_i, [_i, _i, _i, _v, _v, _v]),
    "vcpcu_autotune": (_i, [_v, _v]),
    "vcpcu_autotune_choice": (_i, [_i, _i, _i, _i]),
    "vcpcu_autotune_pick": (_i, [_i, _i, _i, _v, _i, _v, _i, _v, _v, _v]),
    "vcpcu_igemm_batched_dev": (_i, [_i, _v, _i, _i, _v]),
    "vcpcu_batch_graph_create": (_i, [_i, _v, _i, _i, _v, _v]),
    "vcpcu_batch_graph_launch": (_i, [_v, _v]),
    "vcpcu_batch_graph_latencies": (_i, [_v, _v, _v, _v]),
    "vcpcu_batch_graph_destroy": (_i, [_v]),
    "vcpcu_igemm_noalloc_dev": (_i, [_i, _i, _i, _v, _i, _v, _i, _v, _i, _i, _v]),
    "vcpcu_tensor_basis_dev": (_i, [_i, _v, _v, _i, _v, _v, _i, _i, _v, _v, _v, C.c_long, _i,
                                    _i, _v]),
}


def load() -> C.CDLL:
    """Load libvcpcuda.so once; raise if it is absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is not built; run vcp_gb300.build.build() "
                    "(no CPU fallback exists)")
            lib = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
        return _lib


def call(name: str, *args) -> None:
    """Call an int-returning entry point and raise on a non-zero status."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != 0:
        msg = lib.vcpcu_last_error_string().decode(errors="replace")
        raise_for_status(st, f"{name}: {msg}")


def profile(enable: bool) -> None:
    call("vcpcu_profile", 1 if enable else 0)


def profile_read(nphases: int = 5) -> tuple[list[float], int]:
    """(ms per phase [prep, radius 1, radius 2, midpoint GEMM, reassembly],
    tensor flops)."""
    ms = (C.c_double * nphases)()
    fl = C.c_longlong(0)
    call("vcpcu_profile_read", C.cast(ms, C.c_void_p), nphases,
         C.cast(C.pointer(fl), C.c_void_p))
    return list(ms), int(fl.value)


def launch_count() -> int:
    return int(load().vcpcu_launch_count())
