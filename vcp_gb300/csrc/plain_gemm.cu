// plain_gemm.cu -- FP64 CUDA-core GEMMs with per-instruction directed
// rounding: the "plain form" of the verified product.
//
// Result definition (vblas/README.md, "packing layout"; the AVX-512 micro
// kernel vblas/rmatmul_avx512.hpp:195-242 keeps the C tile in registers and
// continues the chain across k blocks): entry C(i,j) is the sequential chain
//     c = +0.0;  for p = 0..K-1:  c = fma_dir(A(i,p), B(p,j), c)
// in ascending p.  Every thread here owns whole C entries and runs exactly
// that chain, so the kernels are bit-identical to vblas rmatmul/udmatmul for
// any tiling.  K tails are padded with +0.0 * +0.0 = +0.0 products, which
// leave every chain value unchanged in all three rounding modes (a -0.0
// accumulator can only arise under round-down, where -0.0 + +0.0 = -0.0).
//
// The interval kernel follows pidblas::mulmm (vcp/pidblas.hpp:239-294): its
// four dgemm_ calls become four chains per entry in one pass over A and B:
//     lo = chain_rd(mA*mB)          (:264-266)
//     up = chain_ru(mA*mB)          (:269-271)
//     t1 = chain_ru((|mA|+rA)*rB)   (:273-279; |mA|+rA rounded up)
//     t2 = chain_ru(rA*|mB|)        (:281)
//     T  = t1 +ru t2 ; up = up +ru T ; lo = lo -rd T   (:283-286)
// with mA, rA, mB, rB from kv-style midrad (pidblas.hpp:43-51).
#include <type_traits>

#include "common.cuh"
#include "plain_gemm.cuh"
#include "swfp.cuh"

namespace vcpcu {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

// Kinds of chains a kernel runs per C entry.
enum Kind { K_RN = 0, K_RU = 1, K_RD = 2, K_UD = 3 };

template <int KIND>
__device__ __forceinline__ double fma_k(double a, double b, double c) {
  if (KIND == K_RU) return __fma_ru(a, b, c);
  if (KIND == K_RD) return __fma_rd(a, b, c);
  return __fma_rn(a, b, c);
}

// One-direction (KIND RN/RU/RD) or up+down (K_UD) point GEMM.
// GEMM naming: C(M x N) = A(M x K) * B(K x N), column-major.
template <int KIND>
__global__ void __launch_bounds__(NT)
point_gemm_kernel(int M, int N, int K, const double* __restrict__ A, long lda,
                  const double* __restrict__ B, long ldb, double* __restrict__ C0,
                  double* __restrict__ C1, long ldc) {
  constexpr int NCH = (KIND == K_UD) ? 2 : 1;
  __shared__ double As[2][BK][BM];
  __shared__ double Bs[2][BK][BN];

  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;

  // loader coordinates
  const int a_i = tid % BM, a_k = tid / BM;        // A: 4 rows of k per pass
  const int b_k = tid % BK, b_j = tid / BK;        // B: 16 columns per pass

  double acc[NCH][4][4];
#pragma unroll
  for (int c = 0; c < NCH; ++c)
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[c][i][j] = 0.0;

  double ra[4], rb[4];
  auto load_tile = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int gi = row0 + a_i, gk = k0 + a_k + 4 * q;
      ra[q] = (gi < M && gk < K) ? A[gi + gk * lda] : 0.0;
      int hk = k0 + b_k, hj = col0 + b_j + 16 * q;
      rb[q] = (hk < K && hj < N) ? B[hk + hj * ldb] : 0.0;
    }
  };
  auto store_tile = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      As[buf][a_k + 4 * q][a_i] = ra[q];
      Bs[buf][b_k][b_j + 16 * q] = rb[q];
    }
  };

  const int nk = (K + BK - 1) / BK;
  load_tile(0);
  store_tile(0);
  __syncthreads();
  for (int t = 0; t < nk; ++t) {
    const int buf = t & 1;
    if (t + 1 < nk) load_tile((t + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[buf][kk][tr + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[buf][kk][tc + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (KIND == K_UD) {
            acc[0][i][j] = __fma_ru(a[i], b[j], acc[0][i][j]);
            acc[NCH - 1][i][j] = __fma_rd(a[i], b[j], acc[NCH - 1][i][j]);
          } else {
            acc[0][i][j] = fma_k<KIND>(a[i], b[j], acc[0][i][j]);
          }
        }
    }
    if (t + 1 < nk) {
      store_tile(buf ^ 1);
    }
    __syncthreads();
  }

#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gi = row0 + tr + 16 * i, gj = col0 + tc + 16 * j;
      if (gi < M && gj < N) {
        C0[gi + gj * ldc] = acc[0][i][j];
        if (KIND == K_UD) C1[gi + gj * ldc] = acc[NCH - 1][i][j];
      }
    }
}

// C = 0 for the n <= 0 (empty inner dimension) case of vblas rmatmul.
__global__ void zero_kernel(int M, int N, double* C, long ldc) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  long total = (long)M * N;
  for (; idx < total; idx += (long)gridDim.x * blockDim.x) {
    long i = idx % M, j = idx / M;
    C[i + j * ldc] = 0.0;
  }
}

}  // namespace

// kv-style midpoint/radius of [lo, up]: m = fl((lo + up) / 2) to nearest
// (halves taken separately when lo + up overflows), r = max(m - lo, up - m)
// rounded up, so that [m - r, m + r] contains [lo, up].  Explicit _rn
// intrinsics keep the compiler from contracting into an FMA.
__device__ __forceinline__ void midrad_dev(double lo, double up, double& m, double& r) {
  double s = __dadd_rn(lo, up);
  if (isfinite(s))
    m = __dmul_rn(s, 0.5);
  else
    m = __dadd_rn(__dmul_rn(lo, 0.5), __dmul_rn(up, 0.5));
  r = fmax(__dsub_ru(m, lo), __dsub_ru(up, m));
}

// Left factor: interval A (m x k, ld in intervals) -> planes mA, pA = |mA| +ru rA, rA
// (ld = M).  Right factor: interval B -> planes mB, rB (ld = K).
// With plus_rad == 0 the middle plane is |mA| itself (the Aᵀ[A] kernel).
__global__ void interval_prep_left(int M, int K, const double* __restrict__ A, long lda,
                                   double* __restrict__ mA, double* __restrict__ pA,
                                   double* __restrict__ rA, int plus_rad = 1) {
  long total = (long)M * K;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long i = idx % M, p = idx / M;
    const double* e = A + 2 * (i + p * lda);
    double m, r;
    midrad_dev(e[0], e[1], m, r);
    mA[idx] = m;
    rA[idx] = r;
    pA[idx] = plus_rad ? __dadd_ru(fabs(m), r) : fabs(m);
  }
}

__global__ void interval_prep_right(int K, int N, const double* __restrict__ B, long ldb,
                                    double* __restrict__ mB, double* __restrict__ rB) {
  long total = (long)K * N;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long p = idx % K, j = idx / K;
    const double* e = B + 2 * (p + j * ldb);
    double m, r;
    midrad_dev(e[0], e[1], m, r);
    mB[idx] = m;
    rB[idx] = r;
  }
}

namespace {

// Fused mid-rad interval GEMM over prepped planes (ld = M for A planes,
// ld = K for B planes).  Writes C as {inf, sup} pairs (ld in intervals).
// Five operand planes are staged per k step, so the k tile is BKI = 8 deep
// (double-buffered: 40 KB of shared memory).
constexpr int BKI = 8;
__global__ void __launch_bounds__(NT)
interval_gemm_kernel(int M, int N, int K, const double* __restrict__ mA,
                     const double* __restrict__ pA, const double* __restrict__ rA,
                     const double* __restrict__ mB, const double* __restrict__ rB,
                     double* __restrict__ C, long ldc) {
  __shared__ double Am[2][BKI][BM], Ap[2][BKI][BM], Ar[2][BKI][BM];
  __shared__ double Bm[2][BKI][BN], Br[2][BKI][BN];

  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  const int a_i = tid % BM, a_k = tid / BM;    // 4 k rows per pass, 2 passes
  const int b_k = tid % BKI, b_j = tid / BKI;  // 32 columns per pass, 2 passes
  constexpr int QA = BKI / (NT / BM), QB = BN / (NT / BKI);

  double lo[4][4], up[4][4], t1[4][4], t2[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) lo[i][j] = up[i][j] = t1[i][j] = t2[i][j] = 0.0;

  double ram[QA], rap[QA], rar[QA], rbm[QB], rbr[QB];
  auto load_tile = [&](int k0) {
#pragma unroll
    for (int q = 0; q < QA; ++q) {
      int gi = row0 + a_i, gk = k0 + a_k + (NT / BM) * q;
      bool ok = gi < M && gk < K;
      long o = gi + (long)gk * M;
      ram[q] = ok ? mA[o] : 0.0;
      rap[q] = ok ? pA[o] : 0.0;
      rar[q] = ok ? rA[o] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      int hk = k0 + b_k, hj = col0 + b_j + (NT / BKI) * q;
      bool okb = hk < K && hj < N;
      long ob = hk + (long)hj * K;
      rbm[q] = okb ? mB[ob] : 0.0;
      rbr[q] = okb ? rB[ob] : 0.0;
    }
  };
  auto store_tile = [&](int buf) {
#pragma unroll
    for (int q = 0; q < QA; ++q) {
      Am[buf][a_k + (NT / BM) * q][a_i] = ram[q];
      Ap[buf][a_k + (NT / BM) * q][a_i] = rap[q];
      Ar[buf][a_k + (NT / BM) * q][a_i] = rar[q];
    }
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      Bm[buf][b_k][b_j + (NT / BKI) * q] = rbm[q];
      Br[buf][b_k][b_j + (NT / BKI) * q] = rbr[q];
    }
  };

  const int nk = (K + BKI - 1) / BKI;
  load_tile(0);
  store_tile(0);
  __syncthreads();
  for (int t = 0; t < nk; ++t) {
    const int buf = t & 1;
    if (t + 1 < nk) load_tile((t + 1) * BKI);
#pragma unroll 2
    for (int kk = 0; kk < BKI; ++kk) {
      double am[4], ap[4], ar[4], bm[4], br[4], bma[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        am[i] = Am[buf][kk][tr + 16 * i];
        ap[i] = Ap[buf][kk][tr + 16 * i];
        ar[i] = Ar[buf][kk][tr + 16 * i];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        bm[j] = Bm[buf][kk][tc + 16 * j];
        br[j] = Br[buf][kk][tc + 16 * j];
        bma[j] = fabs(bm[j]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          lo[i][j] = __fma_rd(am[i], bm[j], lo[i][j]);
          up[i][j] = __fma_ru(am[i], bm[j], up[i][j]);
          t1[i][j] = __fma_ru(ap[i], br[j], t1[i][j]);
          t2[i][j] = __fma_ru(ar[i], bma[j], t2[i][j]);
        }
    }
    if (t + 1 < nk) store_tile(buf ^ 1);
    __syncthreads();
  }

#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gi = row0 + tr + 16 * i, gj = col0 + tc + 16 * j;
      if (gi < M && gj < N) {
        double T = __dadd_ru(t1[i][j], t2[i][j]);
        double u = __dadd_ru(up[i][j], T);
        double l = __dsub_rd(lo[i][j], T);
        double* e = C + 2 * (gi + (long)gj * ldc);
        e[0] = l;
        e[1] = u;
      }
    }
}

// R = Y [C] with imats::mul_m_im's own loop (vcp/imats.hpp:203-213), the
// product the base class runs on its local interval matrices (imats::eigsymge
// forms R = Y (A X - B X Lambda) with it): per entry c = [0, 0], then
// c = c + [y, y] * C(j, k) for j ascending, every step with kv's interval
// operations -- the product as the first smallest of RD(y cl), RD(y cu) and
// the first largest of RU(y cl), RU(y cu) (std::min_element / max_element
// over kv's four candidates), the sum rounded outward.  Eight FP64
// operations per term.  Padding terms are [+0, +0] and leave c unchanged.
__global__ void __launch_bounds__(NT)
imats_mulmm_kernel(int M, int N, int K, const double* __restrict__ Y, long ldy,
                   const double* __restrict__ C, long ldc, double* __restrict__ R, long ldr) {
  __shared__ double Ys[2][BKI][BM], Cl[2][BKI][BN], Cu[2][BKI][BN];
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  const int a_i = tid % BM, a_k = tid / BM;
  const int b_k = tid % BKI, b_j = tid / BKI;
  constexpr int QA = BKI / (NT / BM), QB = BN / (NT / BKI);
  double lo[4][4], up[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) lo[i][j] = up[i][j] = 0.0;
  double ry[QA], rl[QB], ru[QB];
  auto load_tile = [&](int k0) {
#pragma unroll
    for (int q = 0; q < QA; ++q) {
      const int gi = row0 + a_i, gk = k0 + a_k + (NT / BM) * q;
      ry[q] = (gi < M && gk < K) ? Y[gi + (long)gk * ldy] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      const int hk = k0 + b_k, hj = col0 + b_j + (NT / BKI) * q;
      const bool ok = hk < K && hj < N;
      const double* e = C + 2 * (hk + (long)hj * ldc);
      rl[q] = ok ? e[0] : 0.0;
      ru[q] = ok ? e[1] : 0.0;
    }
  };
  auto store_tile = [&](int buf) {
#pragma unroll
    for (int q = 0; q < QA; ++q) Ys[buf][a_k + (NT / BM) * q][a_i] = ry[q];
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      Cl[buf][b_k][b_j + (NT / BKI) * q] = rl[q];
      Cu[buf][b_k][b_j + (NT / BKI) * q] = ru[q];
    }
  };
  const int nk = (K + BKI - 1) / BKI;
  load_tile(0);
  store_tile(0);
  __syncthreads();
  for (int t = 0; t < nk; ++t) {
    const int buf = t & 1;
    if (t + 1 < nk) load_tile((t + 1) * BKI);
#pragma unroll 2
    for (int kk = 0; kk < BKI; ++kk) {
      double y[4], cl[4], cu[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) y[i] = Ys[buf][kk][tr + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        cl[j] = Cl[buf][kk][tc + 16 * j];
        cu[j] = Cu[buf][kk][tc + 16 * j];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const double p1 = __dmul_rd(y[i], cl[j]), p2 = __dmul_rd(y[i], cu[j]);
          const double q1 = __dmul_ru(y[i], cl[j]), q2 = __dmul_ru(y[i], cu[j]);
          lo[i][j] = __dadd_rd(lo[i][j], p2 < p1 ? p2 : p1);
          up[i][j] = __dadd_ru(up[i][j], q1 < q2 ? q2 : q1);
        }
    }
    if (t + 1 < nk) store_tile(buf ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gi = row0 + tr + 16 * i, gj = col0 + tc + 16 * j;
      if (gi < M && gj < N) {
        double* e = R + 2 * (gi + (long)gj * ldr);
        e[0] = lo[i][j];
        e[1] = up[i][j];
      }
    }
}

// [A]ᵀ[A] with pidblas::mulltmm semantics (vcp/pidblas.hpp:296-358) over
// prepped planes: X = Aᵀ (n x k: mX, aX = |mX|, rX), Y = A (k x n: mY, rY).
// Five chains per entry (i, j):
//   lo = RD Σ mX mY, up = RU Σ mX mY          (dsyrk under RD / RU)
//   t1 = RU Σ aX rY   = (|mA|ᵀ rA)(i,j)       (the dgemm temp)
//   t2 = RU Σ rX |mY| = (|mA|ᵀ rA)(j,i)
//   t3 = RU Σ rX rY   = (rAᵀ rA)(i,j)          (dsyrk of rA)
// temp = t1 +ru (t2 +ru t3) for i <= j; C(i,j) = C(j,i) =
// [lo -rd temp, up +ru temp] taken from the upper triangle.
__global__ void __launch_bounds__(NT)
syrk_interval_kernel(int N, int K, const double* __restrict__ mX, const double* __restrict__ aX,
                     const double* __restrict__ rX, const double* __restrict__ mY,
                     const double* __restrict__ rY, double* __restrict__ C, long ldc) {
  __shared__ double Xm[2][BKI][BM], Xa[2][BKI][BM], Xr[2][BKI][BM];
  __shared__ double Ym[2][BKI][BN], Yr[2][BKI][BN];
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  if (col0 + BN <= row0) return;  // tile entirely below the diagonal
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int a_i = tid % BM, a_k = tid / BM;
  const int b_k = tid % BKI, b_j = tid / BKI;
  constexpr int QA = BKI / (NT / BM), QB = BN / (NT / BKI);
  double lo[4][4], up[4][4], t1[4][4], t2[4][4], t3[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) lo[i][j] = up[i][j] = t1[i][j] = t2[i][j] = t3[i][j] = 0.0;
  double ram[QA], raa[QA], rar[QA], rbm[QB], rbr[QB];
  auto load_tile = [&](int k0) {
#pragma unroll
    for (int q = 0; q < QA; ++q) {
      int gi = row0 + a_i, gk = k0 + a_k + (NT / BM) * q;
      bool ok = gi < N && gk < K;
      long o = gi + (long)gk * N;
      ram[q] = ok ? mX[o] : 0.0;
      raa[q] = ok ? aX[o] : 0.0;
      rar[q] = ok ? rX[o] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      int hk = k0 + b_k, hj = col0 + b_j + (NT / BKI) * q;
      bool okb = hk < K && hj < N;
      long ob = hk + (long)hj * K;
      rbm[q] = okb ? mY[ob] : 0.0;
      rbr[q] = okb ? rY[ob] : 0.0;
    }
  };
  auto store_tile = [&](int buf) {
#pragma unroll
    for (int q = 0; q < QA; ++q) {
      Xm[buf][a_k + (NT / BM) * q][a_i] = ram[q];
      Xa[buf][a_k + (NT / BM) * q][a_i] = raa[q];
      Xr[buf][a_k + (NT / BM) * q][a_i] = rar[q];
    }
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      Ym[buf][b_k][b_j + (NT / BKI) * q] = rbm[q];
      Yr[buf][b_k][b_j + (NT / BKI) * q] = rbr[q];
    }
  };
  const int nk = (K + BKI - 1) / BKI;
  load_tile(0);
  store_tile(0);
  __syncthreads();
  for (int t = 0; t < nk; ++t) {
    const int buf = t & 1;
    if (t + 1 < nk) load_tile((t + 1) * BKI);
#pragma unroll 2
    for (int kk = 0; kk < BKI; ++kk) {
      double xm[4], xa[4], xr[4], ym[4], yr[4], ya[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        xm[i] = Xm[buf][kk][tr + 16 * i];
        xa[i] = Xa[buf][kk][tr + 16 * i];
        xr[i] = Xr[buf][kk][tr + 16 * i];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        ym[j] = Ym[buf][kk][tc + 16 * j];
        yr[j] = Yr[buf][kk][tc + 16 * j];
        ya[j] = fabs(ym[j]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          lo[i][j] = __fma_rd(xm[i], ym[j], lo[i][j]);
          up[i][j] = __fma_ru(xm[i], ym[j], up[i][j]);
          t1[i][j] = __fma_ru(xa[i], yr[j], t1[i][j]);
          t2[i][j] = __fma_ru(xr[i], ya[j], t2[i][j]);
          t3[i][j] = __fma_ru(xr[i], yr[j], t3[i][j]);
        }
    }
    if (t + 1 < nk) store_tile(buf ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gi = row0 + tr + 16 * i, gj = col0 + tc + 16 * j;
      if (gi < N && gj < N && gi <= gj) {
        const double temp = __dadd_ru(t1[i][j], __dadd_ru(t2[i][j], t3[i][j]));
        const double u = __dadd_ru(up[i][j], temp);
        const double l = __dsub_rd(lo[i][j], temp);
        double* e = C + 2 * (gi + (long)gj * ldc);
        e[0] = l;
        e[1] = u;
        double* f = C + 2 * (gj + (long)gi * ldc);
        f[0] = l;
        f[1] = u;
      }
    }
}

inline int grid_1d(long total) {
  long b = (total + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

// ---------------------------------------------------------------------------
// Thin right factor (N <= kThinN columns: the matrix-vector products of
// imats::linearsolve, vcp/imats.hpp:305-309, which pdblas hands to dgemv_,
// vcp/pdblas.hpp:96-100).  The tile kernel would spend all but N of its 64
// columns of FP64 work on padding.  Here two lanes own one row of C and run
// its four chains in ascending k: the even lane the two midpoint chains, the
// odd lane the two radius chains.  Both issue the same instructions: the
// round-down chain runs negated as a round-up chain,
// RD(a b + c) = -RU((-a) b + (-c)) (signed zeros included), each lane loads
// its own pair of left operands -- (-mA, mA) or (|mA| +ru rA, rA), written
// by thin_prep_left from A's kv intervals (midrad on the integer pipe,
// sw_midrad, bit-identical to midrad_dev), or formed from a point A -- and
// reads its own copy of B's planes from shared memory (even: mB, mB; odd:
// rB, |mB|), so no lane diverges.  There are only 2 M lanes, each one
// sequential chain: GB300's FP64 unit (one warp-DFMA per 64 cycles per
// sub-partition) bounds the kernel, and the operands are streamed ahead in
// registers so that loads do not add their latency to every step.
constexpr int THIN_KC = 64, THIN_NT = 64;  // THIN_KC a multiple of the prefetch depth

template <int NB, bool A_POINT>
__global__ void __launch_bounds__(THIN_NT)
interval_gemm_thin_kernel(int M, int N, int K, const double* __restrict__ A, long lda,
                          const double* __restrict__ mB, const double* __restrict__ rB,
                          double* __restrict__ C, long ldc) {
  // [parity][k][j] with the odd lanes' copy one double further on (no bank
  // conflict between the two broadcast addresses of a warp)
  constexpr int PLANE = THIN_KC * NB + 1;
  __shared__ double s0[2 * PLANE], s1[2 * PLANE];
  const int t = blockIdx.x * THIN_NT + threadIdx.x;
  const int row = t >> 1;
  const int i = row < M ? row : M - 1;  // lanes past the last row shadow it, store nothing
  const int odd = t & 1;
  const double* y0p = s0 + odd * PLANE;
  const double* y1p = s1 + odd * PLANE;
  double c0[NB], c1[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    c0[j] = odd ? 0.0 : -0.0;  // the even lane's c0 is the negated round-down chain
    c1[j] = 0.0;
  }
  // point A: A[i + k lda]; intervals: the prepared pairs X[k][i][parity]
  constexpr int PF = 16;
  typedef typename std::conditional<A_POINT, double, double2>::type AT;
  const AT* ap = reinterpret_cast<const AT*>(A);
  auto load = [&](int k) -> AT {
    if constexpr (A_POINT) {
      return k < K ? ap[i + (long)k * lda] : 0.0;
    } else {
      return k < K ? ap[2 * ((long)k * M + i) + odd] : make_double2(0.0, 0.0);
    }
  };
  AT cur[PF], nxt[PF];
#pragma unroll
  for (int p = 0; p < PF; ++p) cur[p] = load(p);
  for (int kb = 0; kb < K; kb += PF) {
    const int kbase = kb % THIN_KC;
    if (kbase == 0) {  // stage the next THIN_KC steps of B
      const int kc = min(THIN_KC, K - kb);
      __syncthreads();
      for (int q = threadIdx.x; q < THIN_KC * NB; q += THIN_NT) {
        const int kk = q % THIN_KC, j = q / THIN_KC;
        const bool ok = kk < kc && j < N;
        const double bm = ok ? mB[kb + kk + (long)j * K] : 0.0;
        const double br = ok ? rB[kb + kk + (long)j * K] : 0.0;
        const int o = kk * NB + j;
        s0[o] = bm;
        s1[o] = bm;
        s0[PLANE + o] = br;
        s1[PLANE + o] = sw_double(sw_bits(bm) & 0x7fffffffffffffffULL);
      }
      __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < PF; ++p) nxt[p] = load(kb + PF + p);
#pragma unroll
    for (int p = 0; p < PF; ++p) {
      if (kb + p < K) {
        double x0, x1;
        if constexpr (A_POINT) {  // midrad of [a, a]: (a, +0), |a| +ru 0 = |a|
          x0 = odd ? sw_double(sw_bits(cur[p]) & 0x7fffffffffffffffULL) : sw_neg(cur[p]);
          x1 = odd ? 0.0 : cur[p];
        } else {
          x0 = cur[p].x;
          x1 = cur[p].y;
        }
        const int kk = kbase + p;
#pragma unroll
        for (int j = 0; j < NB; ++j) {
          c0[j] = __fma_ru(x0, y0p[kk * NB + j], c0[j]);
          c1[j] = __fma_ru(x1, y1p[kk * NB + j], c1[j]);
        }
      }
    }
#pragma unroll
    for (int p = 0; p < PF; ++p) cur[p] = nxt[p];
  }
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    const double T = __dadd_ru(c0[j], c1[j]);  // odd lane: t1 +ru t2
    const double To = __shfl_xor_sync(0xffffffffu, T, 1);
    if (!odd && row < M && j < N) {
      double* e = C + 2 * (i + (long)j * ldc);
      e[0] = __dsub_rd(sw_neg(c0[j]), To);
      e[1] = __dadd_ru(c1[j], To);
    }
  }
}

// The left operands of the thin kernel for an interval A (M x K, lda): per
// entry the even lane's pair (-mA, mA) and the odd lane's (|mA| +ru rA, rA),
// X[k][i][parity] (midrad on the integer pipe, many lanes).
__global__ void thin_prep_left(int M, int K, const double* __restrict__ A, long lda,
                               double2* __restrict__ X) {
  const long total = (long)M * K;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const long i = idx % M, k = idx / M;
    const double2 e = reinterpret_cast<const double2*>(A)[i + k * lda];
    double m, r, p;
    sw_midrad(e.x, e.y, m, r, p);
    X[2 * idx] = make_double2(sw_neg(m), m);
    X[2 * idx + 1] = make_double2(p, r);
  }
}

// Planes of the thin right factor (K x N, ld = K): kv midrad of an interval
// B, or the point entries with zero radii (the midrad of [b, b]).
template <bool B_POINT>
__global__ void thin_prep_right(int K, int N, const double* __restrict__ B, long ldb,
                                double* __restrict__ mB, double* __restrict__ rB) {
  const long total = (long)K * N;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const long p = idx % K, j = idx / K;
    if (B_POINT) {
      mB[idx] = B[p + j * ldb];
      rB[idx] = 0.0;
    } else {
      const double* e = B + 2 * (p + j * ldb);
      double m, r;
      midrad_dev(e[0], e[1], m, r);
      mB[idx] = m;
      rB[idx] = r;
    }
  }
}

template <int NB>
void thin_launch(int M, int N, int K, const double* A, long lda, bool a_point,
                 const double* mB, const double* rB, double* C, long ldc, cudaStream_t s) {
  const long threads = 2L * M;
  const int blocks = (int)((threads + THIN_NT - 1) / THIN_NT);
  if (a_point)
    interval_gemm_thin_kernel<NB, true><<<blocks, THIN_NT, 0, s>>>(M, N, K, A, lda, mB, rB, C, ldc);
  else
    interval_gemm_thin_kernel<NB, false><<<blocks, THIN_NT, 0, s>>>(M, N, K, A, lda, mB, rB, C,
                                                                   ldc);
}

}  // namespace

int launch_point_gemm(int M, int N, int K, const double* A, long lda, const double* B,
                      long ldb, double* C0, double* C1, long ldc, int kind,
                      cudaStream_t s) {
  if (M <= 0 || N <= 0) return VCPCU_OK;
  if (K <= 0) {
    zero_kernel<<<grid_1d((long)M * N), 256, 0, s>>>(M, N, C0, ldc);
    VCPCU_LAUNCH_CHECK("zero_kernel");
    if (C1) {
      zero_kernel<<<grid_1d((long)M * N), 256, 0, s>>>(M, N, C1, ldc);
      VCPCU_LAUNCH_CHECK("zero_kernel");
    }
    return VCPCU_OK;
  }
  dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN);
  switch (kind) {
    case PK_UP:
      point_gemm_kernel<K_RU><<<grid, NT, 0, s>>>(M, N, K, A, lda, B, ldb, C0, nullptr, ldc);
      break;
    case PK_DOWN:
      point_gemm_kernel<K_RD><<<grid, NT, 0, s>>>(M, N, K, A, lda, B, ldb, C0, nullptr, ldc);
      break;
    case PK_UPDOWN:
      point_gemm_kernel<K_UD><<<grid, NT, 0, s>>>(M, N, K, A, lda, B, ldb, C0, C1, ldc);
      break;
    default:
      point_gemm_kernel<K_RN><<<grid, NT, 0, s>>>(M, N, K, A, lda, B, ldb, C0, nullptr, ldc);
      break;
  }
  VCPCU_LAUNCH_CHECK("point_gemm_kernel");
  return VCPCU_OK;
}

int launch_interval_gemm_plain(int M, int N, int K, const double* A, long lda,
                               const double* B, long ldb, double* C, long ldc,
                               double* ws, cudaStream_t s) {
  if (N <= kThinN)
    return launch_interval_gemm_thin(M, N, K, A, lda, false, B, ldb, false, C, ldc, ws, s);
  // ws holds 3*M*K + 2*K*N doubles.
  double* mA = ws;
  double* pA = mA + (size_t)M * K;
  double* rA = pA + (size_t)M * K;
  double* mB = rA + (size_t)M * K;
  double* rB = mB + (size_t)K * N;
  interval_prep_left<<<grid_1d((long)M * K), 256, 0, s>>>(M, K, A, lda, mA, pA, rA);
  VCPCU_LAUNCH_CHECK("interval_prep_left");
  interval_prep_right<<<grid_1d((long)K * N), 256, 0, s>>>(K, N, B, ldb, mB, rB);
  VCPCU_LAUNCH_CHECK("interval_prep_right");
  dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN);
  interval_gemm_kernel<<<grid, NT, 0, s>>>(M, N, K, mA, pA, rA, mB, rB, C, ldc);
  VCPCU_LAUNCH_CHECK("interval_gemm_kernel");
  return VCPCU_OK;
}

// (A k x n interval, lda) -> Aᵀ (n x k, ld = n) interval.
__global__ void transpose_interval(int K, int N, const double* __restrict__ A, long lda,
                                   double* __restrict__ At) {
  long total = (long)K * N;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long j = idx % N, p = idx / N;  // At(j, p) = A(p, j), writes coalesced
    const double* e = A + 2 * (p + j * lda);
    At[2 * idx] = e[0];
    At[2 * idx + 1] = e[1];
  }
}

int launch_isyrk_plain(int N, int K, const double* A, long lda, double* C, long ldc, double* ws,
                       cudaStream_t s) {
  // ws: At (2 N K) + mX, aX, rX (3 N K) + mY, rY (2 K N)
  double* At = ws;
  double* mX = At + 2 * (size_t)N * K;
  double* aX = mX + (size_t)N * K;
  double* rX = aX + (size_t)N * K;
  double* mY = rX + (size_t)N * K;
  double* rY = mY + (size_t)N * K;
  if (K > 0) {
    transpose_interval<<<grid_1d((long)N * K), 256, 0, s>>>(K, N, A, lda, At);
    VCPCU_LAUNCH_CHECK("transpose_interval");
    interval_prep_left<<<grid_1d((long)N * K), 256, 0, s>>>(N, K, At, N, mX, aX, rX, 0);
    VCPCU_LAUNCH_CHECK("interval_prep_left");
    interval_prep_right<<<grid_1d((long)K * N), 256, 0, s>>>(K, N, A, lda, mY, rY);
    VCPCU_LAUNCH_CHECK("interval_prep_right");
  }
  dim3 grid((N + BM - 1) / BM, (N + BN - 1) / BN);
  syrk_interval_kernel<<<grid, NT, 0, s>>>(N, K, mX, aX, rX, mY, rY, C, ldc);
  VCPCU_LAUNCH_CHECK("syrk_interval_kernel");
  return VCPCU_OK;
}

size_t isyrk_plain_ws_bytes(int N, int K) { return sizeof(double) * 7 * (size_t)N * K; }

int launch_imats_mulmm(int M, int N, int K, const double* Y, long ldy, const double* C, long ldc,
                       double* R, long ldr, cudaStream_t s) {
  if (M <= 0 || N <= 0) return VCPCU_OK;
  dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN);
  imats_mulmm_kernel<<<grid, NT, 0, s>>>(M, N, K > 0 ? K : 0, Y, ldy, C, ldc, R, ldr);
  VCPCU_LAUNCH_CHECK("imats_mulmm_kernel");
  return VCPCU_OK;
}

size_t interval_gemm_plain_ws_bytes(int M, int N, int K) {
  if (N <= kThinN) return interval_gemm_thin_ws_bytes(M, N, K, false);
  return sizeof(double) * (3 * (size_t)M * K + 2 * (size_t)K * N);
}

int launch_interval_gemm_thin(int M, int N, int K, const double* A, long lda, bool a_point,
                              const double* B, long ldb, bool b_point, double* C, long ldc,
                              double* ws, cudaStream_t s) {
  if (M <= 0 || N <= 0) return VCPCU_OK;
  if (N > kThinN) {
    set_error("interval_gemm_thin: N = %d exceeds %d", N, kThinN);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (K < 0) K = 0;
  double* mB = ws;
  double* rB = mB + (size_t)K * N;
  const double* Al = A;
  long ldl = lda;
  if (!a_point && K > 0) {  // the left operand pairs, after B's planes (16-byte aligned)
    double2* X = reinterpret_cast<double2*>(ws + round_up(2 * (size_t)K * N, 2));
    thin_prep_left<<<grid_1d((long)M * K), 256, 0, s>>>(M, K, A, lda, X);
    VCPCU_LAUNCH_CHECK("thin_prep_left");
    Al = reinterpret_cast<const double*>(X);
    ldl = 0;
  }
  if (K > 0) {
    if (b_point)
      thin_prep_right<true><<<grid_1d((long)K * N), 256, 0, s>>>(K, N, B, ldb, mB, rB);
    else
      thin_prep_right<false><<<grid_1d((long)K * N), 256, 0, s>>>(K, N, B, ldb, mB, rB);
    VCPCU_LAUNCH_CHECK("thin_prep_right");
  }
  if (N == 1)
    thin_launch<1>(M, N, K, Al, ldl, a_point, mB, rB, C, ldc, s);
  else if (N == 2)
    thin_launch<2>(M, N, K, Al, ldl, a_point, mB, rB, C, ldc, s);
  else if (N <= 4)
    thin_launch<4>(M, N, K, Al, ldl, a_point, mB, rB, C, ldc, s);
  else if (N <= 8)
    thin_launch<8>(M, N, K, Al, ldl, a_point, mB, rB, C, ldc, s);
  else
    thin_launch<16>(M, N, K, Al, ldl, a_point, mB, rB, C, ldc, s);
  VCPCU_LAUNCH_CHECK("interval_gemm_thin_kernel");
  return VCPCU_OK;
}

size_t interval_gemm_thin_ws_bytes(int M, int N, int K, bool a_point) {
  const size_t k = K > 0 ? K : 1, b = round_up(2 * k * (N > 0 ? N : 1), 2);
  return sizeof(double) * (b + (a_point ? 0 : 4 * (size_t)(M > 0 ? M : 1) * k));
}

}  // namespace vcpcu
