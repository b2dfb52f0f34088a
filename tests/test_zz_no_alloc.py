"""GPU test of vcpcu_igemm_noalloc_dev, the interval product for callers that
cannot allocate device memory (real-time loops that must not reach
cudaMalloc, which can synchronise the device; processes whose device memory
belongs to another allocator; FFI callers that promise no allocation after
start-up).

It is called through the C ABI and compared with vcpcu_igemm_dev (Ozaki
form, same slice count): the two run the same kernels, so the results must
be bit-identical -- the tolerance of every Ozaki parity test here.  Two calls
in a row with different shapes and data check that the shared static scratch
carries no state from one call into the next.  A problem larger than the
32 MiB static scratch must be rejected, and a non-finite input must be
reported by vcpcu_status exactly as the allocating entry point reports it.

This file sorts last so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from vcp_gb300 import workloads as W
from vcp_gb300.errors import DimensionError, NonFiniteError

pytestmark = pytest.mark.gpu


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def run_both(cuda_lib, m, n, k, slices, seed):
    import torch
    from vcp_gb300 import _lib, pidcuda
    rng = np.random.default_rng(seed)
    A = torch.from_numpy(W.interval_ephi(rng, m, k, 4, 2.0 ** -40)).cuda()
    B = torch.from_numpy(W.interval_ephi(rng, k, n, 4, 2.0 ** -40)).cuda()
    C_ref = torch.full((2 * m * n,), -7.0, dtype=torch.float64, device="cuda")
    C_new = torch.full((2 * m * n,), 3.0, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    pidcuda.mulmm_dev(m, n, k, A, m, B, k, C_ref, m, pidcuda.FORM_OZAKI, slices)
    _lib.call("vcpcu_igemm_noalloc_dev", m, n, k, A.data_ptr(), m, B.data_ptr(), k,
              C_new.data_ptr(), m, slices, s)
    torch.cuda.synchronize()
    _lib.call("vcpcu_status", s)
    return C_ref.cpu().numpy(), C_new.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(cuda_lib):
    ref1, new1 = run_both(cuda_lib, 200, 180, 700, 8, seed=1)
    assert np.array_equal(bits(new1), bits(ref1))
    # second call: a different (smaller) problem over the same static scratch
    ref2, new2 = run_both(cuda_lib, 129, 70, 900, 6, seed=2)
    assert np.array_equal(bits(new2), bits(ref2))
    assert np.all(new2[0::2] <= new2[1::2])


def test_noalloc_rejects_problems_beyond_the_static_scratch(cuda_lib):
    from vcp_gb300 import _lib
    with pytest.raises(DimensionError, match="static scratch"):
        # checked before any pointer is touched
        _lib.call("vcpcu_igemm_noalloc_dev", 4096, 4096, 4096, 16, 4096, 16, 4096, 16, 4096,
                  8, None)


def test_noalloc_reports_nonfinite_input_like_the_allocating_entry_point(cuda_lib):
    import torch
    from vcp_gb300 import _lib
    rng = np.random.default_rng(3)
    m, n, k = 40, 30, 50
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    A[10] = np.nan
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    dC = torch.zeros(2 * m * n, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    _lib.call("vcpcu_igemm_noalloc_dev", m, n, k, dA.data_ptr(), m, dB.data_ptr(), k,
              dC.data_ptr(), m, 8, s)
    torch.cuda.synchronize()
    with pytest.raises(NonFiniteError):
        _lib.call("vcpcu_status", s)
    assert torch.isnan(dC).all().item()
    # the sticky status was taken: a clean call right after reports nothing
    dA = torch.from_numpy(W.interval_ephi(rng, m, k, 4, 2.0 ** -40)).cuda()
    _lib.call("vcpcu_igemm_noalloc_dev", m, n, k, dA.data_ptr(), m, dB.data_ptr(), k,
              dC.data_ptr(), m, 8, s)
    torch.cuda.synchronize()
    _lib.call("vcpcu_status", s)
    assert not torch.isnan(dC).any().item()


# CUmemPool_attribute value of the driver API: the high-water mark of the
# pool's memory in use since its last reset
_CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8


class _DefaultPool:
    """The current device's default stream-ordered pool (where
    cudaMallocAsync takes memory), read through the driver API."""

    def __init__(self):
        import torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        for fn in ("cuDeviceGet", "cuDeviceGetDefaultMemPool", "cuMemPoolSetAttribute",
                   "cuMemPoolGetAttribute"):
            getattr(self.cu, fn).restype = ctypes.c_int
        dev = ctypes.c_int(-1)
        assert self.cu.cuDeviceGet(ctypes.byref(dev), torch.cuda.current_device()) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def reset_high(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, _CU_MEMPOOL_ATTR_USED_MEM_HIGH,
                                             ctypes.byref(zero)) == 0

    def high(self) -> int:
        v = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, _CU_MEMPOOL_ATTR_USED_MEM_HIGH,
                                             ctypes.byref(v)) == 0
        return v.value


def test_noalloc_takes_no_memory_from_the_stream_ordered_pool(cuda_lib):
    """The allocating entry point takes its scratch from the device's
    stream-ordered pool; the no-allocation one must not: the pool's
    high-water mark of memory in use stays where it was across a call, while
    the same product through vcpcu_igemm_dev raises it."""
    import torch
    from vcp_gb300 import _lib, pidcuda
    rng = np.random.default_rng(4)
    m, n, k = 200, 180, 700
    A = torch.from_numpy(W.interval_ephi(rng, m, k, 4, 2.0 ** -40)).cuda()
    B = torch.from_numpy(W.interval_ephi(rng, k, n, 4, 2.0 ** -40)).cuda()
    C = torch.empty(2 * m * n, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream

    def noalloc():
        _lib.call("vcpcu_igemm_noalloc_dev", m, n, k, A.data_ptr(), m, B.data_ptr(), k,
                  C.data_ptr(), m, 8, s)
        torch.cuda.synchronize()
        _lib.call("vcpcu_status", s)

    noalloc()  # the first call on the device looks up the scratch address
    pool = _DefaultPool()
    pool.reset_high()
    base = pool.high()
    noalloc()
    noalloc()
    assert pool.high() == base, "the no-allocation entry point took pool memory"
    pidcuda.mulmm_dev(m, n, k, A, m, B, k, C, m, pidcuda.FORM_OZAKI, 8)
    torch.cuda.synchronize()
    assert pool.high() > base, "the pool check does not see the allocating entry point"
