"""CPU tests of the .vcpmat files (vcp/vcp_portable_fio.hpp) written and read
by libvcpcuda (vcpcu_vcpmat_*, host forms -- no GPU needed):

* every element type, with NaN payloads, infinities, signed zeros and
  subnormals: our files are byte-identical to the reference's own
  vcp::save_portable (compiled from its tree) and each side reads the
  other's files back exactly;
* the CRC-64 trailer equals a bit-by-bit restatement of the reference's
  loop (vcp_portable_fio.hpp:92-108);
* damaged files are rejected by both (vcp::io_error / VCPCU_ERR_IO).
"""
from pathlib import Path

import numpy as np
import pytest

from vcp_gb300 import vcpmat
from vcp_gb300.errors import IOError_

WIDTH = {1: 1, 2: 1, 3: 2, 4: 2, 5: 4}
SHAPES = [(0, 0), (1, 1), (7, 3), (1, 9), (40, 33)]


def crc64_bitwise(data: bytes) -> int:
    poly, crc = 0x42F0E1EBA9EA3693, 0
    for byte in data:
        crc ^= byte << 56
        for _ in range(8):
            crc = ((crc << 1) ^ poly) if crc & (1 << 63) else (crc << 1)
            crc &= (1 << 64) - 1
    return crc


def sample(rng, kind, rows, cols):
    n = rows * cols * WIDTH[kind]
    if kind == 1:
        v = rng.integers(-2 ** 31, 2 ** 31, n, dtype=np.int64).astype(np.int32)
        if n >= 3:
            v[:3] = [-2 ** 31, 2 ** 31 - 1, 0]
        return v
    v = rng.standard_normal(n) * np.ldexp(1.0, rng.integers(-1070, 1000, n))
    specials = np.array([np.nan, np.inf, -np.inf, -0.0, 5e-324, -2.2250738585072014e-308])
    k = min(n, specials.size)
    v[:k] = specials[:k]
    if n > 8:  # a NaN with a payload
        v[7] = np.frombuffer(np.array([0x7FF4000000012345], dtype=np.uint64).tobytes(),
                             dtype=np.float64)[0]
    return v


@pytest.fixture(scope="module")
def ref(oracle):
    import ctypes as C
    R = oracle.ref_lib()
    if R is None:
        from oracle.build import build_reference
        if build_reference() is None:
            pytest.skip("reference sources not mounted")
        R = oracle.ref_lib()
    R.ref_vcpmat_save.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
    R.ref_vcpmat_save.restype = C.c_int
    R.ref_vcpmat_load.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_long]
    R.ref_vcpmat_load.restype = C.c_int
    return R


def ref_load(R, name, kind, cap):
    import ctypes as C
    r, c = C.c_int(-1), C.c_int(-1)
    out = np.zeros(max(cap * WIDTH[kind], 1), dtype=np.int32 if kind == 1 else np.float64)
    st = R.ref_vcpmat_load(name.encode(), kind, C.byref(r), C.byref(c), out.ctypes.data, cap)
    return st, r.value, c.value, out


@pytest.mark.parametrize("kind", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("shape", SHAPES)
def test_files_match_reference_bytes(cuda_lib, ref, tmp_path, kind, shape):
    rows, cols = shape
    data = sample(np.random.default_rng(kind * 100 + rows + cols), kind, rows, cols)
    ours, theirs = str(tmp_path / "ours"), str(tmp_path / "theirs")
    vcpmat.save(ours, data, rows, cols, kind)
    assert ref.ref_vcpmat_save(theirs.encode(), kind, rows, cols,
                               data.ctypes.data if data.size else None) == 0
    b_ours = Path(ours + ".vcpmat").read_bytes()
    b_theirs = Path(theirs + ".vcpmat").read_bytes()
    assert b_ours == b_theirs
    assert int.from_bytes(b_ours[-8:], "little") == crc64_bitwise(b_ours[:-8])
    assert not Path(ours + ".vcpmat.tmp").exists()
    # each side reads the other's file back bit for bit
    got, k, r, c = vcpmat.load(theirs)
    assert (k, r, c) == (vcpmat._NAMES[kind], rows, cols)
    assert got.tobytes() == data.tobytes()
    st, r2, c2, back = ref_load(ref, ours, kind, rows * cols)
    assert st == 0 and (r2, c2) == (rows, cols)
    assert back[: data.size].tobytes() == data.tobytes()


def _damage(path: Path, what: str):
    b = bytearray(path.read_bytes())
    if what == "magic":
        b[0] ^= 1
    elif what == "version":
        b[8] = 3
    elif what == "layout":
        b[16] = 2
    elif what == "reserved":
        b[20] = 1
    elif what == "zero_dim":
        b[24:32] = (0).to_bytes(8, "little")
    elif what == "payload_size":
        b[40] ^= 8
    elif what == "crc":
        b[-1] ^= 0x80
    elif what == "payload_bit":
        b[60] ^= 0x10
    elif what == "truncated":
        b = b[:-9]
    elif what == "trailing":
        b += b"\0"
    path.write_bytes(bytes(b))


@pytest.mark.parametrize("what", ["magic", "version", "layout", "reserved", "zero_dim",
                                  "payload_size", "crc", "payload_bit", "truncated", "trailing"])
def test_damaged_files_rejected_like_reference(cuda_lib, ref, tmp_path, what):
    rows, cols, kind = 6, 5, 3
    data = sample(np.random.default_rng(1), kind, rows, cols)
    name = str(tmp_path / "m")
    vcpmat.save(name, data, rows, cols, kind)
    _damage(Path(name + ".vcpmat"), what)
    st, *_ = ref_load(ref, name, kind, rows * cols)
    assert st == 3, what  # vcp::io_error
    with pytest.raises(IOError_):
        vcpmat.load(name, kind)


def test_type_mismatch_and_missing_file(cuda_lib, ref, tmp_path):
    name = str(tmp_path / "d")
    vcpmat.save(name, np.arange(6, dtype=np.float64), 2, 3, "double")
    with pytest.raises(IOError_):
        vcpmat.load(name, "interval")
    assert ref_load(ref, name, 3, 6)[0] == 3
    with pytest.raises(IOError_):
        vcpmat.info(str(tmp_path / "absent"))
    assert vcpmat.info(name) == ("double", 2, 3)


FIX = Path(__file__).resolve().parent / "golden" / "vcpmat"


@pytest.mark.parametrize("name", ["A", "B", "C", "int32", "double", "dd", "interval_dd"])
def test_reference_fixtures_read_and_rewritten_identically(cuda_lib, tmp_path, name):
    """Files the reference wrote (tests/golden/vcpmat, tests/golden/make_golden.py):
    read, written again, byte-identical (no reference needed)."""
    buf, kind, rows, cols = vcpmat.load(str(FIX / name))
    out = str(tmp_path / name)
    vcpmat.save(out, buf, rows, cols, kind)
    assert Path(out + ".vcpmat").read_bytes() == (FIX / (name + ".vcpmat")).read_bytes()


def test_reference_fixture_product_matches_oracle(cuda_lib, oracle):
    A, _, m, k = vcpmat.load(str(FIX / "A"), "interval")
    B, _, k2, n = vcpmat.load(str(FIX / "B"), "interval")
    C, _, m2, n2 = vcpmat.load(str(FIX / "C"), "interval")
    assert (k2, m2, n2) == (k, m, n)
    assert oracle.pidblas_mulmm(m, n, k, A, B).tobytes() == C.tobytes()
