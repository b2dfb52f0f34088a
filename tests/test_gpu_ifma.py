"""GPU parity of the inf-sup interval FMA (vcpcu_ifma, vcp::ifma) and the
ifma-chain product (vcpcu_igemm_fma, vcp::pidblas_fma::mulmm): bit-identical
to the golden vectors of the reference and to the oracle on every sign case,
enclosing the exact hull, with the edge cases of the reference loop."""
from pathlib import Path

import numpy as np
import pytest

from tests.golden.make_golden import mixed_intervals
from vcp_gb300 import pidcuda
from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def test_ifma_golden_and_oracle(cuda_lib, oracle):
    g = np.load(GOLDEN)
    R = pidcuda.ifma(g["if_A"], g["if_B"], g["if_C"])
    assert np.array_equal(bits(R), bits(g["if_R"]))
    rng = np.random.default_rng(5)
    A, B, C = (mixed_intervals(rng, 50000) for _ in range(3))
    assert np.array_equal(bits(pidcuda.ifma(A, B, C)), bits(oracle.ifma(A, B, C)))


def test_igemm_fma_golden(cuda_lib):
    g = np.load(GOLDEN)
    for idx in range(int(g["n_fm"][0])):
        m, n, k = map(int, g[f"fm{idx}_shape"])
        C = pidcuda.mulmm_fma(g[f"fm{idx}_A"], g[f"fm{idx}_B"], m, n, k)
        assert np.array_equal(bits(C), bits(g[f"fm{idx}_C"])), idx


@pytest.mark.parametrize("shape", [(1, 1, 1), (65, 63, 9), (130, 70, 257), (64, 128, 64)])
def test_igemm_fma_oracle_and_hull(cuda_lib, oracle, shape):
    m, n, k = shape
    rng = np.random.default_rng(sum(shape))
    A, B = mixed_intervals(rng, m * k), mixed_intervals(rng, k * n)
    C = pidcuda.mulmm_fma(A, B, m, n, k)
    assert np.array_equal(bits(C), bits(oracle.pidblas_fma_mulmm(m, n, k, A, B)))
    rows = np.repeat(np.arange(m), n)
    cols = np.tile(np.arange(n), m)
    lo, up = oracle.exact_hull(m, n, k, A, B, rows, cols)
    idx = 2 * (rows + cols * m)
    assert np.all(C[idx] <= lo) and np.all(C[idx + 1] >= up)


def test_igemm_fma_dev_and_edges(cuda_lib, oracle):
    import torch
    m, n, k = 70, 40, 33
    rng = np.random.default_rng(8)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -30)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -30)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.full((2 * m * n,), float("nan"), dtype=torch.float64, device="cuda")
    pidcuda.mulmm_fma_dev(m, n, k, dA, m, dB, k, dC, m)
    torch.cuda.synchronize()
    assert np.array_equal(bits(dC.cpu().numpy()), bits(oracle.pidblas_fma_mulmm(m, n, k, A, B)))
    # inner dimension 0: the chain never starts, C = [0, 0]
    C0 = pidcuda.mulmm_fma(np.empty(0), np.empty(0), 3, 2, 0)
    assert np.all(C0 == 0.0)
