// ifma.cu -- inf-sup interval fused multiply-add (vcp::ifma, vcp/ifma.hpp:48-139)
// and the interval product built on it (vcp::pidblas_fma::mulmm,
// vcp/pidblas_fma.hpp:46-80).
//
// ifma([a], [b], [c]) encloses {x y + z}: the sign cases of [a] and [b]
// select the endpoint products, each formed with one directed fused
// multiply-add onto the matching endpoint of [c]; when both factors contain
// zero, the larger (smaller) of two candidates is kept.  The case order and
// the comparisons are those of the reference's portable branch, so the
// results agree bit for bit (the endpoint tests are done on the bit
// patterns: GB300 issues FP64 comparisons on its narrow FP64 pipe).
//
// The product C = [A] [B] folds ifma over the inner index in ascending
// order, starting from C = [0, 0] -- the loop of pidblas_fma::mulmm -- so
// every entry is the reference's chain.  FP64-bound: 2 to 4 directed FMAs
// per inner step and entry.
#include "common.cuh"
#include "variants.cuh"

namespace vcpcu {

namespace {

__device__ __forceinline__ bool ge0(double x) {  // x >= 0 (true for -0)
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return !(b >> 63) || (b << 1) == 0;
}
__device__ __forceinline__ bool le0(double x) {  // x <= 0 (true for +0)
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) || b == 0;
}

// [resd, resu] = [ad, au] * [bd, bu] + [cd, cu] as vcp::ifma's portable
// branch computes it (inputs finite).
__device__ __forceinline__ void ifma_dev(double au, double ad, double bu, double bd, double cu,
                                         double cd, double& resu, double& resd) {
  double u = 0.0, d = 0.0;
  if (ge0(ad)) {
    if (ge0(bd)) {
      u = __fma_ru(au, bu, cu);
      d = __fma_rd(ad, bd, cd);
    } else if (le0(bd) && ge0(bu)) {
      u = __fma_ru(au, bu, cu);
      d = __fma_rd(au, bd, cd);
    } else if (le0(bu)) {
      u = __fma_ru(ad, bu, cu);
      d = __fma_rd(au, bd, cd);
    }
  } else if (le0(ad) && ge0(au)) {
    if (ge0(bd)) {
      u = __fma_ru(au, bu, cu);
      d = __fma_rd(ad, bu, cd);
    } else if (le0(bd) && ge0(bu)) {
      const double t = __fma_ru(au, bu, cu);
      u = __fma_ru(ad, bd, cu);
      if (u < t) u = t;
      const double t2 = __fma_rd(au, bd, cd);
      d = __fma_rd(ad, bu, cd);
      if (d > t2) d = t2;
    } else if (le0(bu)) {
      u = __fma_ru(ad, bd, cu);
      d = __fma_rd(au, bd, cd);
    }
  } else if (le0(au)) {
    if (ge0(bd)) {
      u = __fma_ru(au, bd, cu);
      d = __fma_rd(ad, bu, cd);
    } else if (le0(bd) && ge0(bu)) {
      u = __fma_ru(ad, bd, cu);
      d = __fma_rd(ad, bu, cd);
    } else if (le0(bu)) {
      u = __fma_ru(ad, bd, cu);
      d = __fma_rd(au, bu, cd);
    }
  }
  resu = u;
  resd = d;
}

// R = ifma(A, B, C) elementwise on kv pairs {inf, sup}; R may alias C.
__global__ void ifma_kernel(long count, const double* __restrict__ A,
                            const double* __restrict__ B, const double* C, double* R) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long)gridDim.x * blockDim.x) {
    const double2 a = reinterpret_cast<const double2*>(A)[i];
    const double2 b = reinterpret_cast<const double2*>(B)[i];
    const double cd = C[2 * i], cu = C[2 * i + 1];
    double u, d;
    ifma_dev(a.y, a.x, b.y, b.x, cu, cd, u, d);
    R[2 * i] = d;
    R[2 * i + 1] = u;
  }
}

// C = fold of ifma over the inner index (ascending) from [0, 0].
// Block: 64 x 64 entries of C, 256 threads with 4 x 4 entries each; k tiles
// of 8 staged (double-buffered) in shared memory as separate inf / sup planes.
constexpr int FM = 64, FN = 64, FK = 8, FT = 256;
__global__ void __launch_bounds__(FT)
igemm_fma_kernel(int M, int N, int K, const double* __restrict__ A, long lda,
                 const double* __restrict__ B, long ldb, double* __restrict__ C, long ldc) {
  __shared__ double Ad[2][FK][FM], Au[2][FK][FM], Bd[2][FK][FN], Bu[2][FK][FN];
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int row0 = blockIdx.x * FM, col0 = blockIdx.y * FN;
  // loaders: A tile 64 x 8 (two entries per thread), B tile 8 x 64 (two per thread)
  const int a_i = tid % FM, a_k = tid / FM;  // a_k in 0..3, second entry at a_k + 4
  const int b_k = tid % FK, b_j = tid / FK;  // b_j in 0..31, second entry at b_j + 32
  double cd[4][4], cu[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) cd[i][j] = cu[i][j] = 0.0;
  double la[2][2], lb[2][2];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int gi = row0 + a_i, gk = k0 + a_k + 4 * q;
      if (gi < M && gk < K) {
        const double2 e = *reinterpret_cast<const double2*>(A + 2 * (gi + (long)gk * lda));
        la[q][0] = e.x;
        la[q][1] = e.y;
      } else {
        la[q][0] = la[q][1] = 0.0;
      }
      const int hk = k0 + b_k, hj = col0 + b_j + 32 * q;
      if (hk < K && hj < N) {
        const double2 e = *reinterpret_cast<const double2*>(B + 2 * (hk + (long)hj * ldb));
        lb[q][0] = e.x;
        lb[q][1] = e.y;
      } else {
        lb[q][0] = lb[q][1] = 0.0;
      }
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      Ad[buf][a_k + 4 * q][a_i] = la[q][0];
      Au[buf][a_k + 4 * q][a_i] = la[q][1];
      Bd[buf][b_k][b_j + 32 * q] = lb[q][0];
      Bu[buf][b_k][b_j + 32 * q] = lb[q][1];
    }
  };
  const int nk = (K + FK - 1) / FK;
  load(0);
  store(0);
  __syncthreads();
  for (int t = 0; t < nk; ++t) {
    const int buf = t & 1;
    if (t + 1 < nk) load((t + 1) * FK);
    const int kmax = min(FK, K - t * FK);  // padding must not take part in the chain
    for (int kk = 0; kk < kmax; ++kk) {
      double ad[4], au[4], bd[4], bu[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        ad[i] = Ad[buf][kk][tr + 16 * i];
        au[i] = Au[buf][kk][tr + 16 * i];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        bd[j] = Bd[buf][kk][tc + 16 * j];
        bu[j] = Bu[buf][kk][tc + 16 * j];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          ifma_dev(au[i], ad[i], bu[j], bd[j], cu[i][j], cd[i][j], cu[i][j], cd[i][j]);
    }
    if (t + 1 < nk) {
      __syncthreads();
      store(buf ^ 1);
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gi = row0 + tr + 16 * i;
    if (gi >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gj = col0 + tc + 16 * j;
      if (gj >= N) continue;
      double* cp = C + 2 * (gi + (long)gj * ldc);
      cp[0] = cd[i][j];
      cp[1] = cu[i][j];
    }
  }
}

}  // namespace

int launch_ifma(long count, const double* A, const double* B, const double* C, double* R,
                cudaStream_t s) {
  if (count <= 0) return VCPCU_OK;
  long blocks = (count + 255) / 256;
  if (blocks > 152L * 32) blocks = 152L * 32;
  ifma_kernel<<<(int)blocks, 256, 0, s>>>(count, A, B, C, R);
  VCPCU_LAUNCH_CHECK("ifma_kernel");
  return VCPCU_OK;
}

int launch_igemm_fma(int M, int N, int K, const double* A, long lda, const double* B, long ldb,
                     double* C, long ldc, cudaStream_t s) {
  dim3 grid((M + FM - 1) / FM, (N + FN - 1) / FN);
  igemm_fma_kernel<<<grid, FT, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc);
  VCPCU_LAUNCH_CHECK("igemm_fma_kernel");
  return VCPCU_OK;
}

}  // namespace vcpcu
