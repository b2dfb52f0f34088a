"""GPU: the failure path of the bounded device waits, without a fault.

vcpcu_selftest_timeout makes one thread wait, with the tensor-core kernels'
own bounded mbarrier wait, on a barrier that nothing arrives on: the wait
gives up, the kernel sets the timeout word and returns, and the status the
library reports is VCPCU_ERR_TIMEOUT.  The status is then clear and the
context still computes (a tensor-core product right after it is
bit-identical to the host model)."""
import numpy as np
import pytest

from vcp_gb300 import _lib, pidcuda
from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_stays_usable(cuda_lib, oracle):
    import time
    import torch
    s = torch.cuda.current_stream()
    lib = _lib.load()
    t0 = time.perf_counter()
    st = lib.vcpcu_selftest_timeout(200_000_000, s.cuda_stream)  # about 0.1 s of waiting
    waited = time.perf_counter() - t0
    assert st == 5, lib.vcpcu_last_error_string()  # VCPCU_ERR_TIMEOUT
    assert b"timed out" in lib.vcpcu_last_error_string()
    assert 0.02 < waited < 30.0
    assert lib.vcpcu_status(s.cuda_stream) == 0  # read and cleared
    m, n, k = 96, 80, 200
    rng = np.random.default_rng(12)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -30)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -30)
    C = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI)
    Cm, _ = oracle.ozaki_igemm(m, n, k, A, B, crt=True)
    assert np.array_equal(C.view(np.int64), Cm.view(np.int64))
