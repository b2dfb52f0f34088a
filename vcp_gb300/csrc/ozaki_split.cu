// ozaki_split.cu -- operand preparation of the Ozaki-form interval product:
// kv-style midrad of every interval entry (the same arithmetic as the plain
// form and as pidblas_assist::midrad, vcp/pidblas.hpp:43-51), per-row /
// per-column power-of-two exponents, and the bf16 digit planes that the
// tcgen05 slice GEMM consumes.
//
// Operands of C = [A]*[B] (A m x k, B k x n, kv layout, column-major):
//   left  (per row i):    mA  -> s   digits, round-to-nearest, exponent Em_i
//                         P = |mA| +ru rA -> sr digits, upward, exponent Ep_i
//                         rA  -> sr digits, upward, exponent Er_i
//                         delta_i = sum over slices and k of |digit|
//   right (per column j): mB  -> s   digits, round-to-nearest, exponent Fm_j
//                         rB  -> sr digits, upward, exponent Fr_j
//                         S = |mB| -> sr digits, upward, exponent Fm_j
//                         beta_j = sum_k |mB(k,j)| rounded upward
// Digit planes are K-major bf16: plane[p][row][k], row < Mp (or Np), k < Kp;
// the padding is zero.
#include "common.cuh"
#include "ozaki.cuh"
#include "ozaki_common.cuh"

namespace vcpcu {

__device__ __forceinline__ void oz_midrad(double lo, double up, double& m, double& r) {
  double s = __dadd_rn(lo, up);
  if (isfinite(s))
    m = __dmul_rn(s, 0.5);
  else
    m = __dadd_rn(__dmul_rn(lo, 0.5), __dmul_rn(up, 0.5));
  r = fmax(__dsub_ru(m, lo), __dsub_ru(up, m));
}

__device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// ---------------------------------------------------------------- left factor
// Row maxima of |mA|, P and rA as double bit patterns (non-negative doubles
// order like their bit patterns).  Block: 32 rows x 8 column phases.
__global__ void oz_rowmax_left(int M, int K, const double* __restrict__ A, long lda,
                               int cols_per_block, unsigned long long* __restrict__ mx,
                               int* __restrict__ flag) {
  __shared__ unsigned long long red[3][32];
  const int lane = threadIdx.x & 31, ph = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  if (threadIdx.x < 32) red[0][lane] = red[1][lane] = red[2][lane] = 0;
  __syncthreads();
  unsigned long long am = 0, ap = 0, ar = 0;
  bool bad = false;
  if (i < M) {
    const int c0 = blockIdx.y * cols_per_block;
    const int c1 = min(K, c0 + cols_per_block);
    for (int c = c0 + ph; c < c1; c += 8) {
      const double* e = A + 2 * (i + (long)c * lda);
      double lo = e[0], up = e[1];
      if (!isfinite(lo) || !isfinite(up)) {
        bad = true;
        continue;
      }
      double m, r;
      oz_midrad(lo, up, m, r);
      double p = __dadd_ru(fabs(m), r);
      am = max(am, dbits(fabs(m)));
      ap = max(ap, dbits(p));
      ar = max(ar, dbits(r));
    }
  }
  if (bad) atomicOr(flag, 1);
  atomicMax(&red[0][lane], am);
  atomicMax(&red[1][lane], ap);
  atomicMax(&red[2][lane], ar);
  __syncthreads();
  if (threadIdx.x < 32 && i < M) {
    atomicMax(&mx[3 * i + 0], red[0][lane]);
    atomicMax(&mx[3 * i + 1], red[1][lane]);
    atomicMax(&mx[3 * i + 2], red[2][lane]);
  }
}

// Exponents from the maxima (one thread per row or column).
__global__ void oz_exponents(int R, const unsigned long long* __restrict__ mx, int nper,
                             int* __restrict__ E) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= R) return;
  for (int t = 0; t < nper; ++t) E[nper * i + t] = oz_exponent(__longlong_as_double((long long)mx[nper * i + t]));
}

// Digit planes of the left factor.  Block: 32 rows x 64 k, 256 threads;
// digits are staged in shared memory and written K-contiguous (transpose).
constexpr int LT_R = 32, LT_K = 64;
__global__ void __launch_bounds__(256)
oz_split_left(int M, int K, int Mp, int Kp, const double* __restrict__ A, long lda, int s,
              int sr, const int* __restrict__ E3, uint16_t* __restrict__ planes_m,
              uint16_t* __restrict__ planes_p, uint16_t* __restrict__ planes_r,
              unsigned long long* __restrict__ delta) {
  extern __shared__ int16_t sd[];  // digits [plane][LT_R][LT_K], values in [-128, 128]
  const int np = s + 2 * sr;
  const int tid = threadIdx.x;
  const int r = tid % LT_R, kph = tid / LT_R;  // 8 k phases
  const int i = blockIdx.y * LT_R + r;
  const int k0 = blockIdx.x * LT_K;
  int Em = OZ_ZERO_EXP, Ep = OZ_ZERO_EXP, Er = OZ_ZERO_EXP;
  if (i < M) {
    Em = E3[3 * i + 0];
    Ep = E3[3 * i + 1];
    Er = E3[3 * i + 2];
  }
  unsigned dsum = 0;
  int d[OZ_MAX_SLICES];
  for (int kk = kph; kk < LT_K; kk += 8) {
    const int k = k0 + kk;
    double m = 0.0, rr = 0.0, p = 0.0;
    if (i < M && k < K) {
      const double* e = A + 2 * (i + (long)k * lda);
      double lo = e[0], up = e[1];
      if (isfinite(lo) && isfinite(up)) {
        oz_midrad(lo, up, m, rr);
        p = __dadd_ru(fabs(m), rr);
      }
    }
    // midpoint digits (two-sided)
    if (Em != OZ_ZERO_EXP && m != 0.0) {
      oz_digits(oz_scaled_int(m, Em, s, 0), s, d);
    } else {
      for (int q = 0; q < s; ++q) d[q] = 0;
    }
    for (int q = 0; q < s; ++q) {
      sd[(q * LT_R + r) * LT_K + kk] = (int16_t)d[q];
      dsum += (unsigned)abs(d[q]);
    }
    // radius factors (upward digits)
    if (Ep != OZ_ZERO_EXP && p != 0.0) {
      oz_digits(oz_scaled_int(p, Ep, sr, 1), sr, d);
    } else {
      for (int q = 0; q < sr; ++q) d[q] = 0;
    }
    for (int q = 0; q < sr; ++q) sd[((s + q) * LT_R + r) * LT_K + kk] = (int16_t)d[q];
    if (Er != OZ_ZERO_EXP && rr != 0.0) {
      oz_digits(oz_scaled_int(rr, Er, sr, 1), sr, d);
    } else {
      for (int q = 0; q < sr; ++q) d[q] = 0;
    }
    for (int q = 0; q < sr; ++q) sd[((s + sr + q) * LT_R + r) * LT_K + kk] = (int16_t)d[q];
  }
  // per-row digit magnitude sum (midpoint slices)
  __shared__ unsigned rsum[LT_R];
  if (tid < LT_R) rsum[tid] = 0;
  __syncthreads();
  atomicAdd(&rsum[r], dsum);
  __syncthreads();
  if (tid < LT_R && blockIdx.y * LT_R + tid < M && rsum[tid])
    atomicAdd(&delta[blockIdx.y * LT_R + tid], (unsigned long long)rsum[tid]);
  // write-out: per plane, 32 rows x 64 k = 2048 bf16; thread -> 8 consecutive k
  const int wr = tid / 8, wk = (tid % 8) * 8;
  const int gi = blockIdx.y * LT_R + wr;
  for (int q = 0; q < np; ++q) {
    uint16_t* base;
    int pl;
    if (q < s) {
      base = planes_m;
      pl = q;
    } else if (q < s + sr) {
      base = planes_p;
      pl = q - s;
    } else {
      base = planes_r;
      pl = q - s - sr;
    }
    uint4 v;
    uint16_t h[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) h[t] = oz_bf16_of_int(sd[(q * LT_R + wr) * LT_K + wk + t]);
    v.x = h[0] | ((uint32_t)h[1] << 16);
    v.y = h[2] | ((uint32_t)h[3] << 16);
    v.z = h[4] | ((uint32_t)h[5] << 16);
    v.w = h[6] | ((uint32_t)h[7] << 16);
    if (gi < Mp) *reinterpret_cast<uint4*>(base + ((size_t)pl * Mp + gi) * Kp + k0 + wk) = v;
  }
}

// --------------------------------------------------------------- right factor
// One block per column j < Np: maxima, beta_j, exponents and digit planes.
__global__ void __launch_bounds__(256)
oz_split_right(int K, int N, int Kp, int Np, const double* __restrict__ B, long ldb, int s,
               int sr, uint16_t* __restrict__ planes_m, uint16_t* __restrict__ planes_r,
               uint16_t* __restrict__ planes_s, int* __restrict__ F2,
               double* __restrict__ beta, int* __restrict__ flag) {
  const int j = blockIdx.x;
  const int tid = threadIdx.x;
  __shared__ unsigned long long smax[2];
  __shared__ double ssum[256];
  if (tid == 0) smax[0] = smax[1] = 0;
  __syncthreads();
  unsigned long long am = 0, ar = 0;
  double bsum = 0.0;
  bool bad = false;
  if (j < N) {
    for (int k = tid; k < K; k += 256) {
      const double* e = B + 2 * (k + (long)j * ldb);
      double lo = e[0], up = e[1];
      if (!isfinite(lo) || !isfinite(up)) {
        bad = true;
        continue;
      }
      double m, r;
      oz_midrad(lo, up, m, r);
      am = max(am, dbits(fabs(m)));
      ar = max(ar, dbits(r));
      bsum = __dadd_ru(bsum, fabs(m));
    }
  }
  if (bad) atomicOr(flag, 1);
  atomicMax(&smax[0], am);
  atomicMax(&smax[1], ar);
  ssum[tid] = bsum;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (tid < w) ssum[tid] = __dadd_ru(ssum[tid], ssum[tid + w]);
    __syncthreads();
  }
  const int Fm = oz_exponent(__longlong_as_double((long long)smax[0]));
  const int Fr = oz_exponent(__longlong_as_double((long long)smax[1]));
  if (tid == 0 && j < N) {
    F2[2 * j + 0] = Fm;
    F2[2 * j + 1] = Fr;
    beta[j] = ssum[0];
  }
  int d[OZ_MAX_SLICES];
  for (int k = tid; k < Kp; k += 256) {
    double m = 0.0, r = 0.0;
    if (j < N && k < K) {
      const double* e = B + 2 * (k + (long)j * ldb);
      double lo = e[0], up = e[1];
      if (isfinite(lo) && isfinite(up)) oz_midrad(lo, up, m, r);
    }
    if (Fm != OZ_ZERO_EXP && m != 0.0)
      oz_digits(oz_scaled_int(m, Fm, s, 0), s, d);
    else
      for (int q = 0; q < s; ++q) d[q] = 0;
    for (int q = 0; q < s; ++q) planes_m[((size_t)q * Np + j) * Kp + k] = oz_bf16_of_int(d[q]);
    if (Fr != OZ_ZERO_EXP && r != 0.0)
      oz_digits(oz_scaled_int(r, Fr, sr, 1), sr, d);
    else
      for (int q = 0; q < sr; ++q) d[q] = 0;
    for (int q = 0; q < sr; ++q) planes_r[((size_t)q * Np + j) * Kp + k] = oz_bf16_of_int(d[q]);
    if (Fm != OZ_ZERO_EXP && m != 0.0)
      oz_digits(oz_scaled_int(fabs(m), Fm, sr, 1), sr, d);
    else
      for (int q = 0; q < sr; ++q) d[q] = 0;
    for (int q = 0; q < sr; ++q) planes_s[((size_t)q * Np + j) * Kp + k] = oz_bf16_of_int(d[q]);
  }
}

// ------------------------------------------------------------------ launchers
int oz_prepare(const OzProblem& pb, const double* A, long lda, const double* B, long ldb,
               OzWorkspace& ws, cudaStream_t st) {
  const int M = pb.M, N = pb.N, K = pb.K;
  VCPCU_CUDA_TRY(cudaMemsetAsync(ws.rowmax, 0, sizeof(unsigned long long) * 3 * (size_t)pb.Mp, st));
  VCPCU_CUDA_TRY(cudaMemsetAsync(ws.delta, 0, sizeof(unsigned long long) * (size_t)pb.Mp, st));
  VCPCU_CUDA_TRY(cudaMemsetAsync(ws.flag, 0, 4 * sizeof(int), st));  // every status word
  if (M > 0 && K > 0) {
    const int cpb = 256;
    dim3 g1((M + 31) / 32, (K + cpb - 1) / cpb);
    oz_rowmax_left<<<g1, 256, 0, st>>>(M, K, A, lda, cpb, ws.rowmax, ws.flag);
    VCPCU_LAUNCH_CHECK("oz_rowmax_left");
  }
  oz_exponents<<<(pb.Mp + 255) / 256, 256, 0, st>>>(pb.Mp, ws.rowmax, 3, ws.E3);
  VCPCU_LAUNCH_CHECK("oz_exponents");
  {
    dim3 g2(pb.Kp / LT_K, pb.Mp / LT_R);
    const size_t shm = sizeof(int16_t) * (size_t)(pb.s + 2 * pb.sr) * LT_R * LT_K;
    VCPCU_CUDA_TRY(cudaFuncSetAttribute(oz_split_left, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)shm));
    oz_split_left<<<g2, 256, shm, st>>>(M, K, pb.Mp, pb.Kp, A, lda, pb.s, pb.sr, ws.E3,
                                        ws.a_mid, ws.a_p, ws.a_r, ws.delta);
    VCPCU_LAUNCH_CHECK("oz_split_left");
  }
  oz_split_right<<<pb.Np, 256, 0, st>>>(K, N, pb.Kp, pb.Np, B, ldb, pb.s, pb.sr, ws.b_mid,
                                        ws.b_r, ws.b_s, ws.F2, ws.beta, ws.flag);
  VCPCU_LAUNCH_CHECK("oz_split_right");
  return VCPCU_OK;
}

}  // namespace vcpcu
