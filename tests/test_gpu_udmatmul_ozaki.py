"""GPU tests of the tensor-core udmatmul (vcpcu_udmatmul_ozaki): CD <= A B <=
CU against the exact dot products (long accumulator), bit-identical to the
host model of the Ozaki form on degenerate intervals (the GPU runs no radius
product for point operands), the slice counts 4..9 of the point-GEMM
workload, the vblas edge cases and the non-finite status."""
import numpy as np
import pytest

from vcp_gb300 import errors, vblas
from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def degenerate(P):
    out = np.empty(2 * P.size)
    out[0::2] = P
    out[1::2] = P
    return out


@pytest.mark.parametrize("phi", [0, 8, 32])
@pytest.mark.parametrize("shape", [(1, 1, 1), (70, 130, 33), (257, 300, 129)])
def test_encloses_and_matches_model(cuda_lib, oracle, phi, shape):
    m, n, k = shape  # vblas naming: A m x n, B n x k
    rng = np.random.default_rng(phi * 7 + m)
    A = W.ephi(rng, m * n, phi)
    B = W.ephi(rng, n * k, phi)
    CU = np.empty(m * k)
    CD = np.empty(m * k)
    vblas.udmatmul_ozaki(m, n, k, A, B, CU, CD)
    rows = np.repeat(np.arange(m), k)
    cols = np.tile(np.arange(k), m)
    dn, up = oracle.exact_dot(m, k, n, A, B, rows, cols)
    idx = rows + cols * m
    assert np.all(CD[idx] <= dn) and np.all(CU[idx] >= up)
    Cm, st = oracle.ozaki_igemm(m, k, n, degenerate(A), degenerate(B), crt=True)
    assert st == 0
    assert np.array_equal(bits(CD), bits(Cm[0::2]))
    assert np.array_equal(bits(CU), bits(Cm[1::2]))


@pytest.mark.parametrize("slices", [4, 5, 6, 7, 8, 9])
def test_slice_counts(cuda_lib, oracle, slices):
    m, n, k = 96, 200, 80
    rng = np.random.default_rng(slices)
    A = W.ephi(rng, m * n, 8)
    B = W.ephi(rng, n * k, 8)
    CU = np.empty(m * k)
    CD = np.empty(m * k)
    vblas.udmatmul_ozaki(m, n, k, A, B, CU, CD, slices)
    rows = np.repeat(np.arange(m), k)
    cols = np.tile(np.arange(k), m)
    dn, up = oracle.exact_dot(m, k, n, A, B, rows, cols)
    idx = rows + cols * m
    assert np.all(CD[idx] <= dn) and np.all(CU[idx] >= up)
    Cm, _ = oracle.ozaki_igemm(m, k, n, degenerate(A), degenerate(B), s=slices, crt=True)
    assert np.array_equal(bits(CD), bits(Cm[0::2]))
    assert np.array_equal(bits(CU), bits(Cm[1::2]))


def test_width_against_fma_chain(cuda_lib):
    """At the default precision (w = 56 bits) the enclosure is no wider than
    the RU/RD FMA-chain pair of udmatmul on well-scaled data."""
    m, n, k = 128, 1024, 128
    rng = np.random.default_rng(5)
    A = W.ephi(rng, m * n, 0)
    B = W.ephi(rng, n * k, 0)
    U1, D1, U2, D2 = (np.empty(m * k) for _ in range(4))
    vblas.udmatmul_ozaki(m, n, k, A, B, U1, D1)
    vblas.udmatmul(m, n, k, A, B, U2, D2)
    assert np.median((U1 - D1) / (U2 - D2)) <= 1.0


def test_edges_and_status(cuda_lib):
    CU = np.full(6, 5.0)
    CD = np.full(6, 5.0)
    vblas.udmatmul_ozaki(2, 0, 3, np.empty(0), np.empty(0), CU, CD)
    assert np.all(CU == 0) and np.all(CD == 0)
    CU[:] = 5.0
    vblas.udmatmul_ozaki(0, 4, 3, np.empty(0), np.empty(12), CU, CD)
    assert np.all(CU == 5.0)
    A = np.ones(4)
    A[2] = np.inf
    with pytest.raises(errors.NonFiniteError):
        vblas.udmatmul_ozaki(2, 2, 2, A, np.ones(4), np.empty(4), np.empty(4))
    with pytest.raises(errors.DimensionError):
        vblas.udmatmul_ozaki(2, 2, 2, np.ones(4), np.ones(4), np.empty(4), np.empty(4), 1)
