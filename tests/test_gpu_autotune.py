"""GPU tests of FORM_AUTO: the calibration returns sane constants, and an AUTO
product is bit-identical to the product in the form the cost model picks,
for single products and for a batch that mixes both forms."""
import numpy as np
import pytest

from vcp_gb300 import batch, pidcuda
from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_autotune_constants(cuda_lib):
    c = pidcuda.autotune()
    assert 2e11 < c["fp64_rate"] < 3e12          # FP64 plain kernel, GB300 ~1.2e12
    assert 1e13 < c["tc_rate"] < 3e15            # bf16 slice GEMMs
    assert c["prep_bw"] > 0 and c["t_launch"] >= 0
    assert pidcuda.autotune_choice(16, 16, 16) == pidcuda.FORM_PLAIN
    assert pidcuda.autotune_choice(4096, 4096, 4096) == pidcuda.FORM_OZAKI


@pytest.mark.parametrize("mnk", [(16, 24, 40), (300, 200, 500), (1030, 900, 1100)])
def test_auto_equals_chosen_form(cuda_lib, mnk):
    import torch
    m, n, k = mnk
    rng = np.random.default_rng(m)
    A = torch.from_numpy(W.interval_uniform(rng, m, k, 1e-12)).cuda()
    B = torch.from_numpy(W.interval_uniform(rng, k, n, 1e-12)).cuda()
    C = torch.empty(2 * m * n, dtype=torch.float64, device="cuda")
    R = torch.empty_like(C)
    pidcuda.mulmm_dev(m, n, k, A, m, B, k, C, m, pidcuda.FORM_AUTO)
    pidcuda.mulmm_dev(m, n, k, A, m, B, k, R, m, pidcuda.autotune_choice(m, n, k))
    torch.cuda.synchronize()
    assert torch.equal(C.view(torch.int64), R.view(torch.int64))


def test_auto_batch_mixes_forms(cuda_lib):
    import torch
    rng = np.random.default_rng(7)
    probs = []
    for (m, n, k) in [(20, 30, 40), (700, 650, 900), (5, 1, 3), (1024, 1024, 1024), (64, 64, 64),
                      (1, 1, 2)]:
        A = torch.from_numpy(W.interval_uniform(rng, m, k, 1e-12)).cuda()
        B = torch.from_numpy(W.interval_uniform(rng, k, n, 1e-12)).cuda()
        C = torch.full((2 * m * n,), float("nan"), dtype=torch.float64, device="cuda")
        probs.append((m, n, k, A, m, B, k, C, m))
    forms = {pidcuda.autotune_choice(p[0], p[1], p[2], batched=True) for p in probs}
    g = batch.BatchGraph(probs, pidcuda.FORM_AUTO)
    g.launch()
    torch.cuda.synchronize()
    for (m, n, k, A, lda, B, ldb, C, ldc) in probs:
        ref = torch.empty_like(C)
        pidcuda.mulmm_dev(m, n, k, A, lda, B, ldb, ref, ldc,
                          pidcuda.autotune_choice(m, n, k, batched=True))
        torch.cuda.synchronize()
        assert torch.equal(C.view(torch.int64), ref.view(torch.int64)), (m, n, k)
    g.close()
    assert forms == {pidcuda.FORM_PLAIN, pidcuda.FORM_OZAKI}
