"""GPU tests of FORM_AUTO: the calibration returns sane constants; an AUTO
product is bit-identical to the product in the form and slice count the
autotuner picks (vcpcu_autotune_pick), for single products and for a batch
that mixes both forms; over inner dimensions {2048, 8192}, exponent spreads
{0, 8, 32} and radius ratios {0, 2^-40, 2^-20} the AUTO enclosures are never
wider than the plain form's (the tuner takes the fast radius products where
they qualify, the exact ones at spread 8 with radii 2^-40 and k = 2048,
where the fast ones leave less margin than its rule asks, and falls back to
the plain form where no slice count qualifies: a 2^64 exponent spread at
k = 2048, radii of 2^-20), and the picks are the ones the host models give
for the same probe."""
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
    form, slices = pidcuda.autotune_pick(A, B, m, n, k)
    assert form == pidcuda.autotune_choice(m, n, k)
    pidcuda.mulmm_dev(m, n, k, A, m, B, k, R, m, form, slices)
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


# (k, phi, radius ratio) -> slice count the probe picks (0: plain form); the
# host models of both forms give these picks for the probe's rows 96..159 and
# columns 0, 4, .., 252 of these seeded 256 x 256 products.
F8 = 8 | pidcuda.SLICES_FAST_RADIUS
AUTO_PICKS = {(2048, 0, 0.0): F8, (2048, 0, 2.0 ** -40): F8, (2048, 0, 2.0 ** -20): 0,
              (2048, 8, 0.0): F8, (2048, 8, 2.0 ** -40): 8, (2048, 8, 2.0 ** -20): 0,
              (2048, 32, 0.0): 0, (2048, 32, 2.0 ** -40): 0, (2048, 32, 2.0 ** -20): 0,
              (8192, 0, 0.0): F8, (8192, 0, 2.0 ** -40): F8, (8192, 0, 2.0 ** -20): 0,
              (8192, 8, 0.0): F8, (8192, 8, 2.0 ** -40): F8, (8192, 8, 2.0 ** -20): 0,
              (8192, 32, 0.0): F8, (8192, 32, 2.0 ** -40): 0, (8192, 32, 2.0 ** -20): 0}


@pytest.mark.parametrize("case", sorted(AUTO_PICKS), ids=lambda c: f"k{c[0]}-phi{c[1]}-r{c[2]:.0e}")
def test_auto_never_wider_than_plain(cuda_lib, case):
    k, phi, rr = case
    m = n = 256
    pidcuda.autotune()  # forget choices other tests made for the same key
    rng = np.random.default_rng(2000 * phi + k + (rr > 0) + (rr > 1e-9))
    A = W.interval_ephi(rng, m, k, phi, rr)
    B = W.interval_ephi(rng, k, n, phi, rr)
    form, slices = pidcuda.autotune_pick(A, B, m, n, k)
    assert slices == AUTO_PICKS[case]
    assert form == (pidcuda.FORM_OZAKI if slices else pidcuda.FORM_PLAIN)
    Ca = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_AUTO)
    Cp = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_PLAIN)
    assert np.all(Ca[1::2] - Ca[0::2] <= Cp[1::2] - Cp[0::2])
    if slices:
        Co = pidcuda.mulmm(A, B, m, n, k, form=pidcuda.FORM_OZAKI, slices=slices)
        assert np.array_equal(Ca.view(np.int64), Co.view(np.int64))


def test_auto_pick_same_from_host_and_device_pointers(cuda_lib):
    import torch
    rng = np.random.default_rng(11)
    m, n, k = 300, 280, 4000
    pidcuda.autotune()
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    h = pidcuda.autotune_pick(A, B, m, n, k)
    d = pidcuda.autotune_pick(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), m, n, k)
    assert h == d == (pidcuda.FORM_OZAKI, F8)
