"""CPU tests of the C ABI boundary: the library loads (no GPU calls) and
exports every function include/vcpcuda.h declares, and the ctypes table of
the Python host side matches the header."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(vcpcu_\w+)\s*\(", text))
    return names


def test_header_declares_core_entry_points():
    names = declared_functions()
    for n in ("vcpcu_rmatmul", "vcpcu_udmatmul", "vcpcu_igemm", "vcpcu_igemm_dev",
              "vcpcu_last_error_string"):
        assert n in names


def test_library_exports_every_declared_symbol(cuda_lib):
    missing = [n for n in sorted(declared_functions()) if not hasattr(cuda_lib, n)]
    assert not missing, missing


def test_ctypes_table_matches_header():
    from vcp_gb300._lib import SIGNATURES
    assert set(SIGNATURES) == declared_functions()


def test_error_mapping():
    import pytest
    from vcp_gb300 import errors
    with pytest.raises(errors.DimensionError):
        errors.raise_for_status(1, "x")
    with pytest.raises(errors.NonFiniteError):
        errors.raise_for_status(3, "x")
    assert issubclass(errors.CudaError, errors.StateError)
    errors.raise_for_status(0, "fine")


def test_autotune_choice_host_model(cuda_lib):
    """The AUTO choice is a host-side cost model: tiny products stay on the
    FP64 plain kernel, large ones go to the tensor-core form.  No GPU call."""
    def choose(m, n, k, batched=0):
        return cuda_lib.vcpcu_autotune_choice(m, n, k, batched)
    assert choose(8, 8, 8) == 0
    assert choose(32, 1, 32) == 0
    assert choose(4096, 4096, 4096) == 1
    assert choose(8192, 8192, 8192) == 1
    # monotone along the diagonal: once Ozaki wins it keeps winning
    picks = [choose(n, n, n) for n in (16, 64, 128, 256, 512, 1024, 2048)]
    assert picks == sorted(picks)
    # without launch costs (a batch) the tensor cores win no later
    for n in (16, 64, 128, 256, 512):
        assert choose(n, n, n, 1) >= choose(n, n, n)


def test_new_entry_points_reject_bad_arguments_without_a_device(cuda_lib):
    """Argument checks of the verification chains, the eigenvalue stages, the
    .vcpmat functions and the timeout self-test run before any device access
    (VCPCU_ERR_INVALID_ARG = 1, VCPCU_ERR_IO = 9)."""
    import ctypes as C
    import numpy as np
    lib = cuda_lib
    a = np.zeros(64)
    p = a.ctypes.data
    # vcpcu_ilss_verify: n, nrhs positive; pointers non-null; form known
    assert lib.vcpcu_ilss_verify(0, 1, p, p, p, p, p, p, 0, 0) == 1
    assert lib.vcpcu_ilss_verify(2, 0, p, p, p, p, p, p, 0, 0) == 1
    assert lib.vcpcu_ilss_verify(2, 1, None, p, p, p, p, p, 0, 0) == 1
    assert lib.vcpcu_ilss_verify(2, 1, p, p, p, p, p, p, 9, 0) == 1
    # the _dev form: leading dimensions below n
    assert lib.vcpcu_ilss_verify_dev(4, 1, p, 3, p, 4, p, 4, p, 4, p, 4, p, 0, 0, None) == 1
    # eigenvalue stages and host form
    assert lib.vcpcu_ieigsymge_stage1_dev(0, p, 1, p, 1, p, 1, p, p, p, 0, 0, None) == 1
    assert lib.vcpcu_ieigsymge_stage2_dev(3, p, p, 2, p, p, p, p, 0, 0, None) == 1
    assert lib.vcpcu_ieigsymge(3, p, p, p, p, None, None, p, p, 0, 0) == 1
    assert lib.vcpcu_eig_merge(-1, p) == 1
    # .vcpmat: unknown type, bad sizes, missing file
    assert lib.vcpcu_vcpmat_save(b"/nonexistent/x", 7, 2, 2, p) == 1
    assert lib.vcpcu_vcpmat_save(b"/nonexistent/x", 2, 0, 3, p) == 1
    t, r, c = C.c_int(), C.c_int(), C.c_int()
    assert lib.vcpcu_vcpmat_info(b"/nonexistent/x", C.byref(t), C.byref(r), C.byref(c)) == 9
    assert lib.vcpcu_vcpmat_save(b"/nonexistent/x", 2, 2, 2, p) == 9  # cannot open
    # the timeout self-test: a limit above 8e9 cycles is refused (no device
    # here: the device check comes first and reports itself)
    assert lib.vcpcu_selftest_timeout(10 ** 10, None) in (1, 2, 6)
