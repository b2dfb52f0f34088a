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
// CRT form: the residues of the w-bit integers A', B' replace the midpoint
// digits, and the sums of the squared low radius digits (P and rA per row,
// rB and |mB| per column) bound the low x low radius pair left out of the
// slice GEMM.
// Digit planes are K-major bf16: plane[p][row][k], row < Mp (or Np), k < Kp;
// the padding is zero.
#include "common.cuh"
#include "ozaki.cuh"
#include "ozaki_common.cuh"
#include "swfp.cuh"

namespace vcpcu {

__device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// bf16 bit pattern of an integer digit |d| <= 256 (exact: the float has at
// most 9 significant bits, so its low 16 bits are zero).  The float is made
// on the FP32 pipe -- 1.5 2^23 + d by adding d to the bit pattern, minus
// 1.5 2^23 (exact for |d| < 2^22) -- instead of an integer conversion, which
// GB300 issues on its narrow FP64 / conversion pipe.
__device__ __forceinline__ uint32_t bf16_bits(int d) {
  return __float_as_uint(__fadd_rn(__int_as_float(0x4B400000 + d), -12582912.0f)) >> 16;
}

template <int S>
__device__ __forceinline__ void digits_of(double x, int E, int up, int (&d)[S]) {
  if (E == OZ_ZERO_EXP || oz_zero(x)) {
#pragma unroll
    for (int q = 0; q < S; ++q) d[q] = 0;
    return;
  }
  if (S <= 7) {
    long long n = oz_scaled_int64(x, E, 8 * S, up);
#pragma unroll
    for (int p = S - 1; p >= 1; --p) {
      const int lo = (int)((unsigned long long)(n + 128) & 255ULL) - 128;
      d[p] = lo;
      n = (n - lo) >> 8;
    }
    d[0] = (int)n;
  } else {
    __int128 n = oz_scaled_int(x, E, S, up);
#pragma unroll
    for (int p = S - 1; p >= 1; --p) {
      const int lo = (int)((unsigned long long)(n + 128) & 255ULL) - 128;
      d[p] = lo;
      n = (n - lo) >> 8;
    }
    d[0] = (int)n;
  }
}

// ---------------------------------------------------------------- left factor
// Pass 1: kv midrad of every entry, stored as the planes mA, rA (column-major,
// ld = ldm), and the row maxima of |mA|, P = |mA| +ru rA and rA as double bit
// patterns (non-negative doubles order like their bit patterns).  One entry
// in four takes the FP64 instructions (sw_midrad_hw, the same bits), the
// others the integer-pipe form: the FP64 pipe then runs beside the integer
// one (at half, the FP64 pipe became the bound).
// Block: 32 rows x 8 column phases over a column range.
__global__ void __launch_bounds__(256)
oz_rowmax_left(int M, int K, const double* __restrict__ A, long lda, int cols_per_block,
               double* __restrict__ mA, double* __restrict__ rA, long ldm,
               unsigned long long* __restrict__ mx, int* __restrict__ flag) {
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
    constexpr int U = 4;  // loads in flight per thread (see oz_colmax_right)
    for (int cb = c0 + ph; cb < c1; cb += 8 * U) {
      double2 e[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int c = cb + 8 * u;
        e[u] = c < c1 ? *reinterpret_cast<const double2*>(A + 2 * (i + (long)c * lda))
                      : make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int c = cb + 8 * u;
        if (c >= c1) break;
        double m = 0.0, r = 0.0, p;
        if (sw_finite(e[u].x) && sw_finite(e[u].y)) {
          if (u == U - 1)
            sw_midrad_hw(e[u].x, e[u].y, m, r, p);
          else
            sw_midrad(e[u].x, e[u].y, m, r, p);
          am = max(am, dbits(oz_abs(m)));
          ap = max(ap, dbits(p));
          ar = max(ar, dbits(r));
        } else {
          bad = true;
        }
        mA[i + (long)c * ldm] = m;
        rA[i + (long)c * ldm] = r;
      }
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
  for (int t = 0; t < nper; ++t)
    E[nper * i + t] = oz_exponent(__longlong_as_double((long long)mx[nper * i + t]));
}

// Pass 2: digit planes of the left factor from the stored mA, rA.  Block:
// 32 rows x 64 k, 256 threads; digits are staged in shared memory and
// written K-contiguous (a transpose), 16 bytes per store.
constexpr int LT_R = 32, LT_K = 64, LT_KS = LT_K + 2;  // padded row: no bank conflicts
template <int S, int SR>
__global__ void __launch_bounds__(256)
oz_split_left(int M, int K, int Mp, int Kp, const double* __restrict__ mA,
              const double* __restrict__ rA, const int* __restrict__ E3,
              uint16_t* __restrict__ planes_m, uint16_t* __restrict__ planes_p,
              uint16_t* __restrict__ planes_r, unsigned long long* __restrict__ delta) {
  extern __shared__ int16_t sd[];  // digits [plane][LT_R][LT_KS], values in [-128, 128]
  constexpr int s = S, sr = SR, np = S + 2 * SR;
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
  int d[S], dr[SR];
  for (int kk = kph; kk < LT_K; kk += 8) {
    const int k = k0 + kk;
    double m = 0.0, rr = 0.0, p = 0.0;
    if (i < M && k < K) {
      m = mA[i + (long)k * M];
      rr = rA[i + (long)k * M];
      p = __dadd_ru(oz_abs(m), rr);
    }
    digits_of<S>(m, Em, 0, d);
#pragma unroll
    for (int q = 0; q < s; ++q) {
      sd[(q * LT_R + r) * LT_KS + kk] = (int16_t)d[q];
      dsum += (unsigned)abs(d[q]);
    }
    digits_of<SR>(p, Ep, 1, dr);
#pragma unroll
    for (int q = 0; q < sr; ++q) sd[((s + q) * LT_R + r) * LT_KS + kk] = (int16_t)dr[q];
    digits_of<SR>(rr, Er, 1, dr);
#pragma unroll
    for (int q = 0; q < sr; ++q) sd[((s + sr + q) * LT_R + r) * LT_KS + kk] = (int16_t)dr[q];
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
    const int16_t* src = sd + (q * LT_R + wr) * LT_KS + wk;
    uint4 v;
    v.x = bf16_bits(src[0]) | (bf16_bits(src[1]) << 16);
    v.y = bf16_bits(src[2]) | (bf16_bits(src[3]) << 16);
    v.z = bf16_bits(src[4]) | (bf16_bits(src[5]) << 16);
    v.w = bf16_bits(src[6]) | (bf16_bits(src[7]) << 16);
    if (gi < Mp) *reinterpret_cast<uint4*>(base + ((size_t)pl * Mp + gi) * Kp + k0 + wk) = v;
  }
}

// --------------------------------------------------------------- right factor
// One block per column j < Np.  Pass 1 (thread t takes k = t, t+256, ...):
// midrad into the planes mB, rB (k contiguous), the column maxima and
// beta_j = RU sum |mB| (per-thread chains, then a pairwise tree).  Pass 2
// (thread t takes 8 consecutive k): digits from the stored planes, 16-byte
// stores.
template <int S, int SR>
__global__ void __launch_bounds__(256)
oz_split_right(int K, int N, int Kp, int Np, const double* __restrict__ B, long ldb,
               double* __restrict__ mBp, double* __restrict__ rBp,
               uint16_t* __restrict__ planes_m, uint16_t* __restrict__ planes_r,
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
  double* mcol = mBp + (size_t)j * Kp;
  double* rcol = rBp + (size_t)j * Kp;
  if (j < N) {
    for (int k = tid; k < K; k += 256) {
      const double2 e = *reinterpret_cast<const double2*>(B + 2 * (k + (long)j * ldb));
      double m = 0.0, r = 0.0, p;
      if (sw_finite(e.x) && sw_finite(e.y)) {
        sw_midrad(e.x, e.y, m, r, p);
        am = max(am, dbits(oz_abs(m)));
        ar = max(ar, dbits(r));
        bsum = __dadd_ru(bsum, fabs(m));
      } else {
        bad = true;
      }
      mcol[k] = m;
      rcol[k] = r;
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
  // pass 2: the planes written above by this block are visible after the
  // barriers of the reduction
  constexpr int s = S, sr = SR;
  int d[S], dr[SR];
  uint32_t hm[S][4], hr[SR][4], hs[SR][4];
  for (int k0 = tid * 8; k0 < Kp; k0 += 256 * 8) {
#pragma unroll
    for (int h = 0; h < 8; ++h) {
      const int k = k0 + h;
      double m = 0.0, r = 0.0;
      if (j < N && k < K) {
        m = mcol[k];
        r = rcol[k];
      }
      digits_of<S>(m, Fm, 0, d);
#pragma unroll
      for (int q = 0; q < s; ++q) {
        const uint32_t b = bf16_bits(d[q]);
        if (h & 1) hm[q][h >> 1] |= b << 16; else hm[q][h >> 1] = b;
      }
      digits_of<SR>(r, Fr, 1, dr);
#pragma unroll
      for (int q = 0; q < sr; ++q) {
        const uint32_t b = bf16_bits(dr[q]);
        if (h & 1) hr[q][h >> 1] |= b << 16; else hr[q][h >> 1] = b;
      }
      digits_of<SR>(oz_abs(m), Fm, 1, dr);
#pragma unroll
      for (int q = 0; q < sr; ++q) {
        const uint32_t b = bf16_bits(dr[q]);
        if (h & 1) hs[q][h >> 1] |= b << 16; else hs[q][h >> 1] = b;
      }
    }
#pragma unroll
    for (int q = 0; q < s; ++q)
      *reinterpret_cast<uint4*>(planes_m + ((size_t)q * Np + j) * Kp + k0) =
          make_uint4(hm[q][0], hm[q][1], hm[q][2], hm[q][3]);
#pragma unroll
    for (int q = 0; q < sr; ++q) {
      *reinterpret_cast<uint4*>(planes_r + ((size_t)q * Np + j) * Kp + k0) =
          make_uint4(hr[q][0], hr[q][1], hr[q][2], hr[q][3]);
      *reinterpret_cast<uint4*>(planes_s + ((size_t)q * Np + j) * Kp + k0) =
          make_uint4(hs[q][0], hs[q][1], hs[q][2], hs[q][3]);
    }
  }
}

// ------------------------------------------------------ CRT form (residues)
// The moduli, largest first (the list the host plan indexes).
#define OZ_MOD_LIST(F)                                                                   \
  F(256), F(255), F(253), F(251), F(247), F(241), F(239), F(233), F(229), F(227), F(223),     \
      F(217), F(211), F(199), F(197), F(193), F(191), F(181), F(179), F(173), F(167), F(163), \
      F(157), F(151), F(149), F(139), F(137), F(131), F(127), F(113), F(109), F(107)

// Residues on the FP32 pipe (the integer multiply pipe is half as wide).
// |a| is cut into b-bit limbs h_t (b = 12; b = 14 for the four-limb form,
// which holds magnitudes <= 2^55; b = 13 for the eight-limb form of the dd
// product, magnitudes < 2^103), exact as floats, and
// x = sum_t h_t c_lt with c_lt = 2^(b t) mod m_l taken in [-m_l/2, m_l/2]:
// |x| <= 128 sum_t |h_t| < 2^23 for every limb form used here (at most 16
// twelve-bit limbs; four 14-bit limbs whose top one is <= 2^13; eight
// 13-bit limbs whose top one is < 2^12), an exact
// float.  One rounded quotient q = rint(RN(x RN(1/m))) then lands within
// |x / m| 2^-23 (1 + 2^-25) < 1 / m of the exact one, so
// r = x - q m (one exact FMA) has |r| <= m/2 + 1 - 1/8, i.e. |r| <= 128:
// a residue of a in the range the slice GEMM's exact chunk sums allow
// (|r_a r_b| <= 2^14 over 1024 terms), and exact in bf16.
__host__ __device__ constexpr int oz_limb_bits(int NL) {
  return NL == 4 ? 14 : (NL == 8 ? 13 : 12);
}
constexpr float oz_limb_c(unsigned long long m, int b, int t) {
  unsigned long long c = 1 % m;
  for (int i = 0; i < t; ++i) c = (c << b) % m;
  return 2 * c > m ? (float)c - (float)m : (float)c;
}
#define OZ_LIMB_ROW(m)                                                                 \
  {oz_limb_c(m, 12, 0), oz_limb_c(m, 12, 1), oz_limb_c(m, 12, 2), oz_limb_c(m, 12, 3),   \
   oz_limb_c(m, 12, 4), oz_limb_c(m, 12, 5), oz_limb_c(m, 12, 6), oz_limb_c(m, 12, 7),   \
   oz_limb_c(m, 12, 8), oz_limb_c(m, 12, 9)}
#define OZ_LIMB14_ROW(m) \
  {oz_limb_c(m, 14, 0), oz_limb_c(m, 14, 1), oz_limb_c(m, 14, 2), oz_limb_c(m, 14, 3)}
#define OZ_LIMB13_ROW(m)                                                                 \
  {oz_limb_c(m, 13, 0), oz_limb_c(m, 13, 1), oz_limb_c(m, 13, 2), oz_limb_c(m, 13, 3),   \
   oz_limb_c(m, 13, 4), oz_limb_c(m, 13, 5), oz_limb_c(m, 13, 6), oz_limb_c(m, 13, 7)}
#define OZ_MODF(m) ((float)(m))
#define OZ_INVF(m) (1.0f / (float)(m))
__constant__ float c_limbf[OZ_MAX_MODULI][10] = {OZ_MOD_LIST(OZ_LIMB_ROW)};
__constant__ float c_limbf14[OZ_MAX_MODULI][4] = {OZ_MOD_LIST(OZ_LIMB14_ROW)};
__constant__ float c_limbf13[OZ_MAX_MODULI][8] = {OZ_MOD_LIST(OZ_LIMB13_ROW)};
__constant__ float c_modf[OZ_MAX_MODULI] = {OZ_MOD_LIST(OZ_MODF)};
__constant__ float c_invf[OZ_MAX_MODULI] = {OZ_MOD_LIST(OZ_INVF)};

// Signed limbs of (neg ? -a : a) as exact floats (b = oz_limb_bits(NL)):
// h_t = sg (2^23 + v_t) - sg 2^23 with sg = -1 or 1.
template <int NL>
__device__ __forceinline__ void limbs12(unsigned long long a, bool neg, float (&h)[NL]) {
  constexpr int B = oz_limb_bits(NL);
  static_assert(NL * B <= 72, "64-bit magnitudes have at most 6 twelve-bit limbs");
  const float sg = neg ? -1.0f : 1.0f;
#pragma unroll
  for (int t = 0; t < NL; ++t) {
    const unsigned v = (unsigned)((a >> (B * t)) & ((1ULL << B) - 1));
    h[t] = __fmaf_rn(sg, __uint_as_float(0x4B000000u | v), -8388608.0f * sg);
  }
}
template <int NL>
__device__ __forceinline__ void limbs12(unsigned __int128 a, bool neg, float (&h)[NL]) {
  constexpr int B = oz_limb_bits(NL);
  const float sg = neg ? -1.0f : 1.0f;
#pragma unroll
  for (int t = 0; t < NL; ++t) {
    const unsigned v = (unsigned)((a >> (B * t)) & ((1ULL << B) - 1));
    h[t] = __fmaf_rn(sg, __uint_as_float(0x4B000000u | v), -8388608.0f * sg);
  }
}

// bf16 patterns of two small integers (exact: at most 8 significant bits) in
// one word, the first in the low half.
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  return __byte_perm(__float_as_uint(a), __float_as_uint(b), 0x7632);
}

// The residues r, |r| <= 128 (see above), of two integers given by their
// signed limbs h0, h1, modulo modulus l, as one word of two bf16 patterns
// (h0's in the low half), all on the FP32 pipe and evaluated pairwise:
// x = h_0 + sum_t h_t c_t by an FMA chain, q = rint(RN(x RN(1/m))) by the
// add and subtract of 1.5 2^23 (round to nearest for |v| < 2^22), and
// r = RN(q (-m) + x), the exact value fma(-q, m, x) would round.
template <int NL>
__device__ __forceinline__ uint32_t res_pair(const float (&h0)[NL], const float (&h1)[NL],
                                             int l) {
  const float m = c_modf[l], inv = c_invf[l];
  const unsigned long long magic = f32x2(12582912.0f, 12582912.0f);
  unsigned long long x = f32x2(h0[0], h1[0]);
#pragma unroll
  for (int t = 1; t < NL; ++t) {
    const float c = NL == 4 ? c_limbf14[l][t] : (NL == 8 ? c_limbf13[l][t] : c_limbf[l][t]);
    x = fma_x2(f32x2(h0[t], h1[t]), f32x2(c, c), x);
  }
  const unsigned long long q = sub_x2(add_x2(mul_x2(x, f32x2(inv, inv)), magic), magic);
  const unsigned long long r = fma_x2(q, f32x2(-m, -m), x);
  return __byte_perm((uint32_t)r, (uint32_t)(r >> 32), 0x7632);
}

// x * 2^e rounded up (up) or down, in steps that stay in the double range.
__device__ __forceinline__ double dev_scale_dir(double x, int e, bool up) {
  while (e > 1023) {
    x = up ? __dmul_ru(x, 0x1p1023) : __dmul_rd(x, 0x1p1023);
    e -= 1023;
  }
  while (e < -1022) {
    x = up ? __dmul_ru(x, 0x1p-1022) : __dmul_rd(x, 0x1p-1022);
    e += 1022;
  }
  const double p = __longlong_as_double((long long)(e + 1023) << 52);
  return up ? __dmul_ru(x, p) : __dmul_rd(x, p);
}

// w-bit integer of x (|x| <= 2^(E-1)): round to nearest even, |result| <= 2^(w-1).
// x 2^(w-E) is formed exactly by power-of-two multiplications (no overflow:
// it stays below 2^(w-1); a subnormal intermediate is below 2^-1022 and
// converts to 0 either way) and converted with one rounding.
__device__ __forceinline__ long long crt_int(double x, int E, int w) {
  if (E == OZ_ZERO_EXP || oz_zero(x)) return 0;
  int s = w - E;
  if (s < -1100) return 0;  // |x| 2^s < 2^-76
  double y = x;
  while (s > 1000) {
    y = __dmul_rn(y, 0x1p1000);
    s -= 1000;
  }
  while (s < -1000) {
    y = __dmul_rn(y, 0x1p-1000);
    s += 1000;
  }
  return __double2ll_rn(__dmul_rn(y, __longlong_as_double((long long)(s + 1023) << 52)));
}

// Stores of a left split's plane tiles (32 rows x 64 k of bf16; lane = row,
// warp q holds k 8q .. 8q + 7 as 16 bytes) through shared memory, so that
// each warp writes 4 rows x 128 contiguous bytes instead of 32 separate
// 16-byte pieces (the planes are k-contiguous, A row-contiguous).  Double
// buffered: one barrier per tile; every thread of the block calls put() the
// same number of times.
struct TileStore {
  uint4 (*T)[32][9];  // [2][32 rows][8 chunks + 1 pad]: conflict-free both ways
  int buf;
  __device__ __forceinline__ void put(uint4 v, uint16_t* tile, int Kp) {
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    T[buf][lane][wq] = v;
    __syncthreads();
    const int r = threadIdx.x >> 3, c = threadIdx.x & 7;
    *reinterpret_cast<uint4*>(tile + (size_t)r * Kp + 8 * c) = T[buf][r][c];
    buf ^= 1;
  }
};

// Left factor, CRT form: residues of A' (L planes) + radius digits, and
// sum_k |A'(i,k)| split as (|A'| >> 32, |A'| & 0xffffffff) sums; the sums
// of the squared low digits of P and rA in asum[4 i + 2], asum[4 i + 3].
// Block: 32 rows x 64 k; lane = row, warp q takes k0 + 8q .. k0 + 8q + 7, so
// the loads of mA / rA are coalesced across the warp; each lane's 8 bf16
// (16 bytes) per plane go out through shared memory (TileStore).
// X = mA and rA are the stored midrad planes (ld ldx).  Planes rows are
// rowbase + i (stacked problems), pstride elements apart; E3 and asum point
// at row 0 of this problem.
// rowmax != null (grouped products): the exponents come from the row maxima
// here, and the blocks of the first k range store them in E3 for the
// reassembly (no separate exponent pass); else they are read from E3.
template <int SR, int NL>
__device__ __forceinline__ void split_left_crt_body(int bx, int by, int M, int K, int Kp,
                                                    size_t pstride, int rowbase,
                                                    const double* __restrict__ X,
                                                    const double* __restrict__ rA, long ldx,
                                                    int L, int w, int* __restrict__ E3,
                                                    uint16_t* __restrict__ planes_m,
                                                    uint16_t* __restrict__ planes_p,
                                                    uint16_t* __restrict__ planes_r,
                                                    unsigned long long* __restrict__ asum,
                                                    const unsigned long long* __restrict__ rowmax =
                                                        nullptr) {
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const int i = by * 32 + lane;
  const int k0 = bx * 64 + wq * 8;
  int Em = OZ_ZERO_EXP, Ep = OZ_ZERO_EXP, Er = OZ_ZERO_EXP;
  if (i < M) {
    if (rowmax) {
      Em = oz_exponent(__longlong_as_double((long long)rowmax[3 * i + 0]));
      Ep = oz_exponent(__longlong_as_double((long long)rowmax[3 * i + 1]));
      Er = oz_exponent(__longlong_as_double((long long)rowmax[3 * i + 2]));
      if (bx == 0 && wq == 0) {
        E3[3 * i + 0] = Em;
        E3[3 * i + 1] = Ep;
        E3[3 * i + 2] = Er;
      }
    } else {
      Em = E3[3 * i + 0];
      Ep = E3[3 * i + 1];
      Er = E3[3 * i + 2];
    }
  }
  __shared__ uint4 tile_smem[2][32][9];
  TileStore ts{tile_smem, 0};
  const size_t tile0 = (size_t)(rowbase + by * 32) * Kp + bx * 64;
  // the warp's 8 k past K, or all 32 rows past M: zero planes, nothing to
  // compute (the stores still go through the tile, every thread calls put)
  const bool pad = k0 >= K || by * 32 >= M;
  long long a[8];
  unsigned long long shi = 0, slo = 0;
  uint32_t qp = 0, qr = 0;  // sums of the squared low radius digits (< 2^18 per lane)
  {
    // radius digit planes first, so that the doubles die before the residues
    uint32_t hp[SR][4] = {}, hr[SR][4] = {};
#pragma unroll
    for (int t = 0; t < 8; ++t) a[t] = 0;
#pragma unroll
    for (int t = 0; t < 8; t += 2) {
      if (pad) break;
      int d0[SR], d1[SR], e0[SR], e1[SR];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int k = k0 + t + u;
        double m = 0.0, r = 0.0, p = 0.0;
        if (i < M && k < K) {
          m = X[i + (long)k * ldx];
          r = rA[i + (long)k * ldx];
          p = __dadd_ru(oz_abs(m), r);
        }
        a[t + u] = crt_int(m, Em, w);
        digits_of<SR>(p, Ep, 1, u ? d1 : d0);
        digits_of<SR>(r, Er, 1, u ? e1 : e0);
      }
      qp += (uint32_t)(d0[SR - 1] * d0[SR - 1] + d1[SR - 1] * d1[SR - 1]);
      qr += (uint32_t)(e0[SR - 1] * e0[SR - 1] + e1[SR - 1] * e1[SR - 1]);
#pragma unroll
      for (int q = 0; q < SR; ++q) {
        hp[q][t / 2] = bf16_bits(d0[q]) | (bf16_bits(d1[q]) << 16);
        hr[q][t / 2] = bf16_bits(e0[q]) | (bf16_bits(e1[q]) << 16);
      }
    }
#pragma unroll
    for (int q = 0; q < SR; ++q) {
      ts.put(make_uint4(hp[q][0], hp[q][1], hp[q][2], hp[q][3]), planes_p + q * pstride + tile0,
             Kp);
      ts.put(make_uint4(hr[q][0], hr[q][1], hr[q][2], hr[q][3]), planes_r + q * pstride + tile0,
             Kp);
    }
  }
  float hl[8][NL];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const unsigned long long ua = (unsigned long long)(a[t] < 0 ? -a[t] : a[t]);
    shi += ua >> 32;
    slo += ua & 0xffffffffULL;
    limbs12<NL>(ua, a[t] < 0, hl[t]);
  }
  __shared__ unsigned long long red[2][32];
  __shared__ uint32_t redq[2][32];
  if (threadIdx.x < 32) {
    red[0][lane] = red[1][lane] = 0;
    redq[0][lane] = redq[1][lane] = 0u;
  }
  __syncthreads();
  atomicAdd(&red[0][lane], shi);
  atomicAdd(&red[1][lane], slo);
  if (qp) atomicAdd(&redq[0][lane], qp);
  if (qr) atomicAdd(&redq[1][lane], qr);
  __syncthreads();
  if (threadIdx.x < 32 && i < M) {
    atomicAdd(&asum[4 * i + 0], red[0][lane]);
    atomicAdd(&asum[4 * i + 1], red[1][lane]);
    if (redq[0][lane]) atomicAdd(&asum[4 * i + 2], (unsigned long long)redq[0][lane]);
    if (redq[1][lane]) atomicAdd(&asum[4 * i + 3], (unsigned long long)redq[1][lane]);
  }
#pragma unroll
  for (int l = 0; l < OZ_MAX_MODULI_128; ++l) {
    if (l >= L) break;
    uint32_t h[4] = {0u, 0u, 0u, 0u};
    if (!pad) {
#pragma unroll
      for (int t = 0; t < 8; t += 2)
        h[t / 2] = res_pair<NL>(hl[t], hl[t + 1], l);
    }
    ts.put(make_uint4(h[0], h[1], h[2], h[3]), planes_m + l * pstride + tile0, Kp);
  }
}

// One row range of the left factor: rows [0, M) of this launch are rows
// rowbase.. of the planes (pstride elements apart); mA / rA (ld ldx), E3
// and asum point at the range's first row.
template <int SR, int NL>
__global__ void __launch_bounds__(256, 4)
oz_split_left_crt(int M, int K, int Kp, size_t pstride, int rowbase,
                  const double* __restrict__ mA, const double* __restrict__ rA, long ldx, int L,
                  int w, int* __restrict__ E3, uint16_t* __restrict__ planes_m,
                  uint16_t* __restrict__ planes_p, uint16_t* __restrict__ planes_r,
                  unsigned long long* __restrict__ asum) {
  split_left_crt_body<SR, NL>(blockIdx.x, blockIdx.y, M, K, Kp, pstride, rowbase, mA, rA, ldx,
                              L, w, E3, planes_m, planes_p, planes_r, asum);
}

// ---------------------------------------------------------- grouped products
__device__ __forceinline__ int g_find(const int* __restrict__ prefix, int nprob, int x) {
  int lo = 0, hi = nprob - 1;  // largest p with prefix[p] <= x
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ unsigned long long g_timer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Row maxima of every problem of a bucket (no midrad planes are kept: the
// left split repeats the midrad); the first block of a problem to run
// stamps its start.
__global__ void __launch_bounds__(256)
oz_rowmax_left_g(const __grid_constant__ OzGBucket b) {
  const int p = g_find(b.blk_rowmax, b.nprob, blockIdx.x);
  const OzGProb& q = b.probs[p];
  const int nbx = (q.m + 31) / 32;
  const int local = blockIdx.x - b.blk_rowmax[p];
  if (threadIdx.x == 0 && b.t_first) atomicMin(&b.t_first[q.orig], g_timer());
  __shared__ unsigned long long red[3][32];
  const int lane = threadIdx.x & 31, ph = threadIdx.x >> 5;
  const int i = (local % nbx) * 32 + lane;
  if (threadIdx.x < 32) red[0][lane] = red[1][lane] = red[2][lane] = 0;
  __syncthreads();
  unsigned long long am = 0, ap = 0, ar = 0;
  bool bad = false;
  if (i < q.m) {
    const int c0 = (local / nbx) * 256;
    const int c1 = min(q.k, c0 + 256);
    const size_t row = (size_t)(q.rowoff + i);
    for (int c = c0 + ph, it = 0; c < c1; c += 8, ++it) {
      const double2 e = *reinterpret_cast<const double2*>(q.A + 2 * (i + (long)c * q.lda));
      double m = 0.0, r = 0.0, pp;
      if (sw_finite(e.x) && sw_finite(e.y)) {
        if ((it & 3) == 3)  // one entry in four on the FP64 pipe (see oz_rowmax_left)
          sw_midrad_hw(e.x, e.y, m, r, pp);
        else
          sw_midrad(e.x, e.y, m, r, pp);
        am = max(am, dbits(oz_abs(m)));
        ap = max(ap, dbits(pp));
        ar = max(ar, dbits(r));
      } else {
        bad = true;
      }
      // stored for the split (column-major over the stacked rows)
      b.midA[row + (size_t)c * b.Mtot] = m;
      b.radA[row + (size_t)c * b.Mtot] = r;
    }
  }
  if (bad) atomicOr(&b.flag[4 * p], 1);
  atomicMax(&red[0][lane], am);
  atomicMax(&red[1][lane], ap);
  atomicMax(&red[2][lane], ar);
  __syncthreads();
  if (threadIdx.x < 32 && i < q.m) {
    unsigned long long* mx = b.rowmax + 3 * (size_t)(q.rowoff + i);
    atomicMax(&mx[0], red[0][lane]);
    atomicMax(&mx[1], red[1][lane]);
    atomicMax(&mx[2], red[2][lane]);
  }
}

template <int NL>
__global__ void __launch_bounds__(256, 3) oz_split_left_crt_g(const __grid_constant__ OzGBucket b) {
  const int p = g_find(b.blk_split, b.nprob, blockIdx.x);
  const OzGProb& q = b.probs[p];
  const int nbx = b.Kp / 64;
  const int local = blockIdx.x - b.blk_split[p];
  const size_t pstride = (size_t)b.Mtot * b.Kp;
  split_left_crt_body<2, NL>(local % nbx, local / nbx, q.m, q.k, b.Kp, pstride, q.rowoff,
                             b.midA + q.rowoff, b.radA + q.rowoff, b.Mtot, q.L, q.w,
                             b.E3 + 3 * (size_t)q.rowoff, b.planesA,
                             b.planesA + (size_t)b.Lmax * pstride,
                             b.planesA + (size_t)(b.Lmax + 2) * pstride,
                             b.asum + 4 * (size_t)q.rowoff, b.rowmax + 3 * (size_t)q.rowoff);
}

// Warp reductions of 64-bit maxima and sums.
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
    v = u > v ? u : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// KPL consecutive bf16 (KPL = 2, 4 or 8: 4, 8 or 16 bytes) in one store.
template <int KPL>
__device__ __forceinline__ void store_bf16s(uint16_t* dst, const uint32_t (&h)[KPL / 2]) {
  if constexpr (KPL == 8)
    *reinterpret_cast<uint4*>(dst) = make_uint4(h[0], h[1], h[2], h[3]);
  else if constexpr (KPL == 4)
    *reinterpret_cast<uint2*>(dst) = make_uint2(h[0], h[1]);
  else
    *reinterpret_cast<uint32_t*>(dst) = h[0];
}

// Grouped right factor in three passes, as for one product.  Pass 1: one
// warp per stacked column (8 per block): midrad stored as midB / radB
// ([Ntot][Kp]), the column maxima and exponents, the column sums cleared;
// padding columns get the zero exponent.
__global__ void __launch_bounds__(256) oz_colmax_right_g(const __grid_constant__ OzGBucket b) {
  const int lane = threadIdx.x & 31;
  const int jst = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (jst >= b.Ntot) return;  // whole warps only
  const int p = b.col_prob[jst];
  const OzGProb& q = b.probs[p];
  const int j = jst - q.coloff, K = q.k;
  unsigned long long am = 0, ar = 0;
  bool bad = false;
  if (j < q.n) {
    const double* bcol = q.B + 2 * (long)j * q.ldb;
    double* mcol = b.midB + (size_t)jst * b.Kp;
    double* rcol = b.radB + (size_t)jst * b.Kp;
    for (int k = lane, it = 0; k < K; k += 32, ++it) {
      const double2 e = *reinterpret_cast<const double2*>(bcol + 2 * k);
      double m = 0.0, r = 0.0;
      if (sw_finite(e.x) && sw_finite(e.y)) {
        double pp;
        if ((it & 3) == 3)  // one entry in four on the FP64 pipe (see oz_rowmax_left)
          sw_midrad_hw(e.x, e.y, m, r, pp);
        else
          sw_midrad(e.x, e.y, m, r, pp);
        am = max(am, dbits(oz_abs(m)));
        ar = max(ar, dbits(r));
      } else {
        bad = true;
      }
      mcol[k] = m;
      rcol[k] = r;
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&b.flag[4 * p], 1);
  am = warp_max_u64(am);
  ar = warp_max_u64(ar);
  if (lane == 0) {
    b.F2[2 * jst + 0] = j < q.n ? oz_exponent(__longlong_as_double((long long)am)) : OZ_ZERO_EXP;
    b.F2[2 * jst + 1] = j < q.n ? oz_exponent(__longlong_as_double((long long)ar)) : OZ_ZERO_EXP;
    b.bsum[4 * jst + 0] = b.bsum[4 * jst + 1] = 0;
    b.bsum[4 * jst + 2] = b.bsum[4 * jst + 3] = 0;
  }
}

// Pass 2: residue and radius-digit planes.  Block: 8 stacked columns x
// 32 KPL k; warp q takes column 8 bx + q, lane t the KPL consecutive k of
// 32 KPL by + KPL t (KPL = 2, 4, 8 by the bucket's Kp, so that short
// columns keep the lanes busy); padding (columns past n, k past K) is
// written as zeros without computing; sum_k |B'| accumulates per column.
template <int NL, int KPL>
__global__ void __launch_bounds__(256) oz_split_right2_g(const __grid_constant__ OzGBucket b) {
  const int lane = threadIdx.x & 31;
  const int jst = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int k0 = (blockIdx.y * 32 + lane) * KPL;
  if (jst >= b.Ntot) return;  // whole warps only (no barrier below)
  const int p = b.col_prob[jst];
  const OzGProb& q = b.probs[p];
  const int j = jst - q.coloff, K = q.k, Kp = b.Kp, L = q.L, w = q.w;
  const size_t pstride = (size_t)b.Ntot * Kp;
  uint16_t* planes_m = b.planesB;
  uint16_t* planes_r = b.planesB + (size_t)b.Lmax * pstride;
  uint16_t* planes_s = b.planesB + (size_t)(b.Lmax + 2) * pstride;
  constexpr int HW = KPL / 2;  // 32-bit words per lane and plane
  unsigned long long shi = 0, slo = 0;
  uint32_t qr = 0, qs = 0;  // sums of the squared low digits of rB, |mB|
  if (k0 < Kp) {
    const size_t off = (size_t)jst * Kp + k0;
    if (j >= q.n || k0 >= K) {  // padding: zeros, nothing to compute
      const uint32_t zero[HW] = {};
#pragma unroll
      for (int qq = 0; qq < 2; ++qq) {
        store_bf16s<KPL>(planes_r + qq * pstride + off, zero);
        store_bf16s<KPL>(planes_s + qq * pstride + off, zero);
      }
      for (int l = 0; l < L; ++l) store_bf16s<KPL>(planes_m + l * pstride + off, zero);
    } else {
      const int Fm = b.F2[2 * jst], Fr = b.F2[2 * jst + 1];
      const double* mcol = b.midB + (size_t)jst * Kp;
      const double* rcol = b.radB + (size_t)jst * Kp;
      float hl[KPL][NL];
      uint32_t hr[2][HW], hs[2][HW];
#pragma unroll
      for (int t = 0; t < KPL; t += 2) {
        int d0[2], d1[2], e0[2], e1[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int k = k0 + t + u;
          double m = 0.0, r = 0.0;
          if (k < K) {
            m = mcol[k];
            r = rcol[k];
          }
          const long long bb = crt_int(m, Fm, w);
          const unsigned long long ub = (unsigned long long)(bb < 0 ? -bb : bb);
          shi += ub >> 32;
          slo += ub & 0xffffffffULL;
          limbs12<NL>(ub, bb < 0, hl[t + u]);
          digits_of<2>(r, Fr, 1, u ? d1 : d0);
          digits_of<2>(oz_abs(m), Fm, 1, u ? e1 : e0);
        }
        qr += (uint32_t)(d0[1] * d0[1] + d1[1] * d1[1]);
        qs += (uint32_t)(e0[1] * e0[1] + e1[1] * e1[1]);
#pragma unroll
        for (int qq = 0; qq < 2; ++qq) {
          hr[qq][t / 2] = bf16_bits(d0[qq]) | (bf16_bits(d1[qq]) << 16);
          hs[qq][t / 2] = bf16_bits(e0[qq]) | (bf16_bits(e1[qq]) << 16);
        }
      }
#pragma unroll
      for (int qq = 0; qq < 2; ++qq) {
        store_bf16s<KPL>(planes_r + qq * pstride + off, hr[qq]);
        store_bf16s<KPL>(planes_s + qq * pstride + off, hs[qq]);
      }
#pragma unroll
      for (int l = 0; l < OZ_MAX_MODULI_128; ++l) {
        if (l >= L) break;
        uint32_t h[HW];
#pragma unroll
        for (int t = 0; t < KPL; t += 2)
          h[t / 2] = res_pair<NL>(hl[t], hl[t + 1], l);
        store_bf16s<KPL>(planes_m + l * pstride + off, h);
      }
    }
  }
  shi = warp_sum_u64(shi);
  slo = warp_sum_u64(slo);
  qr = __reduce_add_sync(0xffffffffu, qr);
  qs = __reduce_add_sync(0xffffffffu, qs);
  if (lane == 0) {
    if (shi | slo) {
      atomicAdd(&b.bsum[4 * jst + 0], shi);
      atomicAdd(&b.bsum[4 * jst + 1], slo);
    }
    if (qr) atomicAdd(&b.bsum[4 * jst + 2], (unsigned long long)qr);
    if (qs) atomicAdd(&b.bsum[4 * jst + 3], (unsigned long long)qs);
  }
}

// Pass 3: beta_j = RU((sum_k |B'| + ceil(K/2)) 2^(Fm - w)) per stacked column.
__global__ void oz_beta_right_g(const __grid_constant__ OzGBucket b) {
  const int jst = blockIdx.x * blockDim.x + threadIdx.x;
  if (jst >= b.Ntot) return;
  const OzGProb& q = b.probs[b.col_prob[jst]];
  const int j = jst - q.coloff, Fm = b.F2[2 * jst];
  double bj = 0.0;
  if (j < q.n && Fm != OZ_ZERO_EXP) {
    const double v = __fma_ru((double)b.bsum[4 * jst], 0x1p32,
                              (double)(b.bsum[4 * jst + 1] + (unsigned long long)(q.k + 1) / 2));
    bj = dev_scale_dir(v, Fm - q.w, true);
  }
  b.beta[jst] = bj;
}

int oz_gprep(const OzGBucket& b, int nblk_rowmax, int nblk_split, int wmax, cudaStream_t st) {
  if (nblk_rowmax > 0) {
    oz_rowmax_left_g<<<nblk_rowmax, 256, 0, st>>>(b);
    VCPCU_LAUNCH_CHECK("oz_rowmax_left_g");
  }
  // |A'|, |B'| <= 2^(w-1): four 14-bit limbs up to w = 56, six 12-bit limbs
  // up to w = 73; lanes of the right split take 2, 4 or 8 consecutive k so
  // that short columns keep the warp busy
  oz_colmax_right_g<<<(b.Ntot + 7) / 8, 256, 0, st>>>(b);
  VCPCU_LAUNCH_CHECK("oz_colmax_right_g");
  const int kpl = b.Kp <= 64 ? 2 : (b.Kp <= 128 ? 4 : 8);
  const dim3 g2((b.Ntot + 7) / 8, (b.Kp + 32 * kpl - 1) / (32 * kpl));
#define OZ_GRIGHT(NL)                                             \
  do {                                                            \
    if (kpl == 2)                                                 \
      oz_split_right2_g<NL, 2><<<g2, 256, 0, st>>>(b);            \
    else if (kpl == 4)                                            \
      oz_split_right2_g<NL, 4><<<g2, 256, 0, st>>>(b);            \
    else                                                          \
      oz_split_right2_g<NL, 8><<<g2, 256, 0, st>>>(b);            \
  } while (0)
  if (wmax <= 56) {
    oz_split_left_crt_g<4><<<nblk_split, 256, 0, st>>>(b);
    VCPCU_LAUNCH_CHECK("oz_split_left_crt_g");
    OZ_GRIGHT(4);
  } else {
    oz_split_left_crt_g<6><<<nblk_split, 256, 0, st>>>(b);
    VCPCU_LAUNCH_CHECK("oz_split_left_crt_g");
    OZ_GRIGHT(6);
  }
#undef OZ_GRIGHT
  VCPCU_LAUNCH_CHECK("oz_split_right2_g");
  // (the exponents of the left factor come from its split)
  oz_beta_right_g<<<(b.Ntot + 255) / 256, 256, 0, st>>>(b);
  VCPCU_LAUNCH_CHECK("oz_beta_right_g");
  return VCPCU_OK;
}

// ------------------------------------------------------------------ launchers
template <int S, int SR>
int launch_splits(const OzProblem& pb, const double* B, long ldb, OzWorkspace& ws,
                  cudaStream_t st) {
  dim3 g2(pb.Kp / LT_K, pb.Mp / LT_R);
  const size_t shm = sizeof(int16_t) * (size_t)(S + 2 * SR) * LT_R * LT_KS;
  VCPCU_CUDA_TRY(cudaFuncSetAttribute(oz_split_left<S, SR>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  oz_split_left<S, SR><<<g2, 256, shm, st>>>(pb.M, pb.K, pb.Mp, pb.Kp, ws.midA, ws.radA, ws.E3,
                                             ws.a_mid, ws.a_p, ws.a_r, ws.delta);
  VCPCU_LAUNCH_CHECK("oz_split_left");
  oz_split_right<S, SR><<<pb.Np, 256, 0, st>>>(pb.K, pb.N, pb.Kp, pb.Np, B, ldb, ws.midB,
                                               ws.radB, ws.b_mid, ws.b_r, ws.b_s, ws.F2,
                                               ws.beta, ws.flag);
  VCPCU_LAUNCH_CHECK("oz_split_right");
  return VCPCU_OK;
}

// ------------------------------------------- right factor, CRT form, 2 passes
// Pass 1: one warp per column (8 per block): kv midrad of the column, stored
// as the planes mB, rB ([cols][Kp], k contiguous), the column maxima of
// |mB| and rB and their exponents (zero exponent for padding columns);
// clears the column's sums of |B'|.  Columns are colbase + j of F2 / bsum.
__global__ void __launch_bounds__(256)
oz_colmax_right(int K, int N, int Kp, int cols, int colbase, const double* __restrict__ B,
                long ldb, double* __restrict__ mB, double* __restrict__ rB,
                int* __restrict__ F2, unsigned long long* __restrict__ bsum,
                int* __restrict__ flag) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (j >= cols) return;  // whole warps only
  unsigned long long am = 0, ar = 0;
  bool bad = false;
  if (j < N) {
    const double* bcol = B + 2 * (long)j * ldb;
    double* mcol = mB + (size_t)j * Kp;
    double* rcol = rB + (size_t)j * Kp;
    // four loads in flight per lane before they are used: with one warp per
    // column a launch over a narrow column block has few warps to hide the
    // latency with (the midrad's out-of-line FP64 fallback keeps the
    // compiler from hoisting loads across iterations by itself)
    constexpr int U = 4;
    for (int k0 = lane; k0 < K; k0 += 32 * U) {
      double2 e[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int k = k0 + 32 * u;
        e[u] = k < K ? *reinterpret_cast<const double2*>(bcol + 2 * k) : make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int k = k0 + 32 * u;
        if (k >= K) break;
        double m = 0.0, r = 0.0;
        if (sw_finite(e[u].x) && sw_finite(e[u].y)) {
          double p;
          if (u == U - 1)
            sw_midrad_hw(e[u].x, e[u].y, m, r, p);
          else
            sw_midrad(e[u].x, e[u].y, m, r, p);
          am = max(am, dbits(oz_abs(m)));
          ar = max(ar, dbits(r));
        } else {
          bad = true;
        }
        mcol[k] = m;
        rcol[k] = r;
      }
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flag, 1);
  am = warp_max_u64(am);
  ar = warp_max_u64(ar);
  if (lane == 0) {
    const int jst = colbase + j;
    F2[2 * jst + 0] = j < N ? oz_exponent(__longlong_as_double((long long)am)) : OZ_ZERO_EXP;
    F2[2 * jst + 1] = j < N ? oz_exponent(__longlong_as_double((long long)ar)) : OZ_ZERO_EXP;
    bsum[4 * jst + 0] = bsum[4 * jst + 1] = 0;
    bsum[4 * jst + 2] = bsum[4 * jst + 3] = 0;
  }
}

// Pass 2 -> residue planes of B' = round(mB 2^(w - Fm)) and the radius
// digit planes of rB and |mB|.  Block: 8 columns x 256 k; warp q takes column
// 8 by + q, lane t the 8 consecutive k of 256 bx + 8 t .. + 7 (2 KB of the
// stored mB and rB read contiguously per warp, 512 contiguous bytes written
// per plane); sum_k |B'| accumulates per column.
template <int NL>
__global__ void __launch_bounds__(256)
oz_split_right_crt2(int K, int N, int Kp, int cols, int colbase, size_t pstride,
                    const double* __restrict__ mB, const double* __restrict__ rB, int L, int w,
                    const int* __restrict__ F2, uint16_t* __restrict__ planes_m,
                    uint16_t* __restrict__ planes_r, uint16_t* __restrict__ planes_s,
                    unsigned long long* __restrict__ bsum) {
  constexpr int SR = 2;
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int k0 = blockIdx.x * 256 + 8 * lane;
  if (j >= cols) return;  // whole warps only (no barrier below)
  const int jst = colbase + j;
  const int Fm = F2[2 * jst], Fr = F2[2 * jst + 1];
  const double* mcol = mB + (size_t)j * Kp;
  const double* rcol = rB + (size_t)j * Kp;
  unsigned long long shi = 0, slo = 0;
  uint32_t qr = 0, qs = 0;  // sums of the squared low digits of rB, |mB|
  if (k0 < Kp) {
    const size_t off = (size_t)jst * Kp + k0;
    float hl[8][NL];
    uint32_t hr[SR][4], hs[SR][4];
#pragma unroll
    for (int t = 0; t < 8; t += 2) {
      int d0[SR], d1[SR], e0[SR], e1[SR];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int k = k0 + t + u;
        double m = 0.0, r = 0.0;
        if (j < N && k < K) {
          m = mcol[k];
          r = rcol[k];
        }
        const long long bb = crt_int(m, Fm, w);
        const unsigned long long ub = (unsigned long long)(bb < 0 ? -bb : bb);
        shi += ub >> 32;
        slo += ub & 0xffffffffULL;
        limbs12<NL>(ub, bb < 0, hl[t + u]);
        digits_of<SR>(r, Fr, 1, u ? d1 : d0);
        digits_of<SR>(oz_abs(m), Fm, 1, u ? e1 : e0);
      }
      qr += (uint32_t)(d0[SR - 1] * d0[SR - 1] + d1[SR - 1] * d1[SR - 1]);
      qs += (uint32_t)(e0[SR - 1] * e0[SR - 1] + e1[SR - 1] * e1[SR - 1]);
#pragma unroll
      for (int q = 0; q < SR; ++q) {
        hr[q][t / 2] = bf16_bits(d0[q]) | (bf16_bits(d1[q]) << 16);
        hs[q][t / 2] = bf16_bits(e0[q]) | (bf16_bits(e1[q]) << 16);
      }
    }
#pragma unroll
    for (int q = 0; q < SR; ++q) {
      *reinterpret_cast<uint4*>(planes_r + q * pstride + off) =
          make_uint4(hr[q][0], hr[q][1], hr[q][2], hr[q][3]);
      *reinterpret_cast<uint4*>(planes_s + q * pstride + off) =
          make_uint4(hs[q][0], hs[q][1], hs[q][2], hs[q][3]);
    }
#pragma unroll
    for (int l = 0; l < OZ_MAX_MODULI_128; ++l) {
      if (l >= L) break;
      uint32_t h[4];
#pragma unroll
      for (int t = 0; t < 8; t += 2)
        h[t / 2] = res_pair<NL>(hl[t], hl[t + 1], l);
      *reinterpret_cast<uint4*>(planes_m + l * pstride + off) = make_uint4(h[0], h[1], h[2], h[3]);
    }
  }
  shi = warp_sum_u64(shi);
  slo = warp_sum_u64(slo);
  qr = __reduce_add_sync(0xffffffffu, qr);
  qs = __reduce_add_sync(0xffffffffu, qs);
  if (lane == 0) {
    if (shi | slo) {
      atomicAdd(&bsum[4 * jst + 0], shi);
      atomicAdd(&bsum[4 * jst + 1], slo);
    }
    if (qr) atomicAdd(&bsum[4 * jst + 2], (unsigned long long)qr);
    if (qs) atomicAdd(&bsum[4 * jst + 3], (unsigned long long)qs);
  }
}

// beta_j = RU((sum_k |B'| + ceil(K/2)) 2^(Fm - w)) >= sum_k |mB(k, j)|.
__global__ void oz_beta_right(int K, int N, int cols, int colbase, int w,
                              const int* __restrict__ F2,
                              const unsigned long long* __restrict__ bsum,
                              double* __restrict__ beta) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  const int jst = colbase + j, Fm = F2[2 * jst];
  double bj = 0.0;
  if (j < N && Fm != OZ_ZERO_EXP) {
    const double v = __fma_ru((double)bsum[4 * jst], 0x1p32,
                              (double)(bsum[4 * jst + 1] + (unsigned long long)(K + 1) / 2));
    bj = dev_scale_dir(v, Fm - w, true);
  }
  beta[jst] = bj;
}

int oz_prepare_left_begin(const OzProblem& pb, OzWorkspace& ws, cudaStream_t st) {
  VCPCU_CUDA_TRY(cudaMemsetAsync(ws.rowmax, 0, sizeof(unsigned long long) * 3 * (size_t)pb.Mp, st));
  VCPCU_CUDA_TRY(cudaMemsetAsync(ws.delta, 0, sizeof(unsigned long long) * (size_t)pb.Mp, st));
  VCPCU_CUDA_TRY(cudaMemsetAsync(ws.flag, 0, 4 * sizeof(int), st));  // every status word
  if (pb.crt)
    VCPCU_CUDA_TRY(cudaMemsetAsync(ws.asum, 0, sizeof(unsigned long long) * 4 * (size_t)pb.Mp, st));
  return VCPCU_OK;
}

int oz_prepare_left_rowmax(const OzProblem& pb, const double* A, long lda, int k0, int k1,
                           OzWorkspace& ws, cudaStream_t st) {
  const int M = pb.M, kc = k1 - k0;
  if (M <= 0 || kc <= 0) return VCPCU_OK;
  const int cpb = 256;
  dim3 g1((M + 31) / 32, (kc + cpb - 1) / cpb);
  oz_rowmax_left<<<g1, 256, 0, st>>>(M, kc, A + 2 * (long)k0 * lda, lda, cpb,
                                     ws.midA + (size_t)k0 * M, ws.radA + (size_t)k0 * M, M,
                                     ws.rowmax, ws.flag);
  VCPCU_LAUNCH_CHECK("oz_rowmax_left");
  return VCPCU_OK;
}

namespace {
// Residue and radius-digit planes (CRT form) of rows [i0, i0 + rows) of the
// left factor, rows a multiple of 32 (padding rows at the end of A give zero
// planes); the exponents of those rows are set.
int split_left_rows(const OzProblem& pb, int i0, int rows, OzWorkspace& ws, cudaStream_t st) {
  if (pb.sr != 2) {
    set_error("Ozaki form: radius slice count %d is not built (2 is)", pb.sr);
    return VCPCU_ERR_UNSUPPORTED;
  }
  if (rows <= 0) return VCPCU_OK;
  const int mv = pb.M - i0 < rows ? (pb.M - i0 > 0 ? pb.M - i0 : 0) : rows;  // valid rows
  const size_t pstride = (size_t)pb.Mp * pb.Kp;
  dim3 g2(pb.Kp / 64, rows / 32);
  const double* mA = ws.midA + i0;
  const double* rA = ws.radA + i0;
  int* E3 = ws.E3 + 3 * (size_t)i0;
  unsigned long long* asum = ws.asum + 4 * (size_t)i0;
  // |A'| <= 2^(w-1): four 14-bit limbs up to w = 56, five 12-bit limbs up to
  // w = 61, six up to 73
  if (pb.w <= 56)
    oz_split_left_crt<2, 4><<<g2, 256, 0, st>>>(mv, pb.K, pb.Kp, pstride, i0, mA, rA, pb.M, pb.L,
                                                pb.w, E3, ws.a_mid, ws.a_p, ws.a_r, asum);
  else if (pb.w <= 61)
    oz_split_left_crt<2, 5><<<g2, 256, 0, st>>>(mv, pb.K, pb.Kp, pstride, i0, mA, rA, pb.M, pb.L,
                                                pb.w, E3, ws.a_mid, ws.a_p, ws.a_r, asum);
  else
    oz_split_left_crt<2, 6><<<g2, 256, 0, st>>>(mv, pb.K, pb.Kp, pstride, i0, mA, rA, pb.M, pb.L,
                                                pb.w, E3, ws.a_mid, ws.a_p, ws.a_r, asum);
  VCPCU_LAUNCH_CHECK("oz_split_left_crt");
  return VCPCU_OK;
}
}  // namespace

int oz_prepare_left_finish(const OzProblem& pb, OzWorkspace& ws, cudaStream_t st) {
  oz_exponents<<<(pb.Mp + 255) / 256, 256, 0, st>>>(pb.Mp, ws.rowmax, 3, ws.E3);
  VCPCU_LAUNCH_CHECK("oz_exponents");
  if (pb.sr != 2) {
    set_error("Ozaki form: radius slice count %d is not built (2 is)", pb.sr);
    return VCPCU_ERR_UNSUPPORTED;
  }
  if (!pb.crt) return VCPCU_OK;  // the slice form splits both factors in launch_splits
  return split_left_rows(pb, 0, pb.Mp, ws, st);
}

int oz_prepare_left_rows(const OzProblem& pb, const double* A, long lda, int i0, int rows,
                         OzWorkspace& ws, cudaStream_t st) {
  const int mv = pb.M - i0 < rows ? (pb.M - i0 > 0 ? pb.M - i0 : 0) : rows;
  if (mv > 0 && pb.K > 0) {
    const int cpb = 256;
    dim3 g1((mv + 31) / 32, (pb.K + cpb - 1) / cpb);
    oz_rowmax_left<<<g1, 256, 0, st>>>(mv, pb.K, A + 2 * (long)i0, lda, cpb, ws.midA + i0,
                                       ws.radA + i0, pb.M, ws.rowmax + 3 * (size_t)i0, ws.flag);
    VCPCU_LAUNCH_CHECK("oz_rowmax_left");
  }
  oz_exponents<<<(rows + 255) / 256, 256, 0, st>>>(rows, ws.rowmax + 3 * (size_t)i0, 3,
                                                   ws.E3 + 3 * (size_t)i0);
  VCPCU_LAUNCH_CHECK("oz_exponents");
  return split_left_rows(pb, i0, rows, ws, st);
}

int oz_prepare_right_crt(const OzProblem& pb, const double* B, long ldb, OzWorkspace& ws,
                         cudaStream_t st, int colbase, int cols, size_t pstride) {
  if (cols < 0) cols = pb.Np;
  if (!pstride) pstride = (size_t)pb.Np * pb.Kp;
  const int nv = pb.N - colbase < cols ? (pb.N - colbase > 0 ? pb.N - colbase : 0) : cols;
  if (cols <= 0) return VCPCU_OK;
  const double* Bc = B + 2 * (size_t)colbase * ldb;
  oz_colmax_right<<<(cols + 7) / 8, 256, 0, st>>>(pb.K, nv, pb.Kp, cols, colbase, Bc, ldb,
                                                  ws.midB, ws.radB, ws.F2, ws.bsum, ws.flag);
  VCPCU_LAUNCH_CHECK("oz_colmax_right");
  dim3 g((pb.Kp + 255) / 256, (cols + 7) / 8);
  // |B'| <= 2^(w-1): four 14-bit limbs up to w = 56, five 12-bit limbs up to
  // w = 61, six up to 73
#define OZ_RIGHT_CRT(NL)                                                                       \
  oz_split_right_crt2<NL><<<g, 256, 0, st>>>(pb.K, nv, pb.Kp, cols, colbase, pstride, ws.midB, \
                                             ws.radB, pb.L, pb.w, ws.F2, ws.b_mid, ws.b_r,      \
                                             ws.b_s, ws.bsum)
  if (pb.w <= 56)
    OZ_RIGHT_CRT(4);
  else if (pb.w <= 61)
    OZ_RIGHT_CRT(5);
  else
    OZ_RIGHT_CRT(6);
#undef OZ_RIGHT_CRT
  VCPCU_LAUNCH_CHECK("oz_split_right_crt2");
  oz_beta_right<<<(cols + 255) / 256, 256, 0, st>>>(pb.K, nv, cols, colbase, pb.w, ws.F2,
                                                    ws.bsum, ws.beta);
  VCPCU_LAUNCH_CHECK("oz_beta_right");
  return VCPCU_OK;
}

int oz_prepare(const OzProblem& pb, const double* A, long lda, const double* B, long ldb,
               OzWorkspace& ws, cudaStream_t st) {
  int st_ = oz_prepare_left_begin(pb, ws, st);
  if (!st_) st_ = oz_prepare_left_rowmax(pb, A, lda, 0, pb.K, ws, st);
  if (!st_) st_ = oz_prepare_left_finish(pb, ws, st);
  if (st_) return st_;
  if (pb.crt) return oz_prepare_right_crt(pb, B, ldb, ws, st);
  switch (pb.s) {
#define OZ_SPLIT_CASE(S)                                                          \
  case S:                                                                         \
    st_ = launch_splits<S, 2>(pb, B, ldb, ws, st);                                \
    break;
    OZ_SPLIT_CASE(2) OZ_SPLIT_CASE(3) OZ_SPLIT_CASE(4) OZ_SPLIT_CASE(5) OZ_SPLIT_CASE(6)
    OZ_SPLIT_CASE(7) OZ_SPLIT_CASE(8) OZ_SPLIT_CASE(9) OZ_SPLIT_CASE(10) OZ_SPLIT_CASE(11)
    OZ_SPLIT_CASE(12)
#undef OZ_SPLIT_CASE
    default:
      set_error("Ozaki form: slice count %d outside [2, 12]", pb.s);
      return VCPCU_ERR_INVALID_ARG;
  }
  return st_;
}

// ------------------------------------------------------------ dd (pddcuda)
// w-bit integer of a dd value hi + lo against exponent E: the two words are
// scaled and rounded to integers separately (|error| <= 1 unit).
__device__ __forceinline__ __int128 dd_int(double hi, double lo, int E, int w) {
  if (E == OZ_ZERO_EXP) return 0;
  __int128 a = 0;
  if (!oz_zero(hi)) a += oz_scaled_int_bits(hi, E, w, 0);
  if (!oz_zero(lo)) a += oz_scaled_int_bits(lo, E, w, 0);
  return a;
}

// Row maxima of |hi| of a dd matrix (kv pairs {a1, a2}, column-major).
__global__ void __launch_bounds__(256)
dd_rowmax(int M, int K, const double* __restrict__ A, long lda, int cols_per_block,
          unsigned long long* __restrict__ mx, int* __restrict__ flag) {
  __shared__ unsigned long long red[32];
  const int lane = threadIdx.x & 31, ph = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  if (threadIdx.x < 32) red[lane] = 0;
  __syncthreads();
  unsigned long long am = 0;
  bool bad = false;
  if (i < M) {
    const int c0 = blockIdx.y * cols_per_block, c1 = min(K, c0 + cols_per_block);
    for (int c = c0 + ph; c < c1; c += 8) {
      const double2 e = *reinterpret_cast<const double2*>(A + 2 * (i + (long)c * lda));
      if (isfinite(e.x) && isfinite(e.y))
        am = max(am, dbits(oz_abs(e.x)));
      else
        bad = true;
    }
  }
  if (bad) atomicOr(flag, 1);
  atomicMax(&red[lane], am);
  __syncthreads();
  if (threadIdx.x < 32 && i < M) atomicMax(&mx[i], red[lane]);
}

// Exponents of the dd form: one bit of headroom over max |hi| so that
// |hi + lo| <= 2^(E-1).
__global__ void dd_exponents(int R, const unsigned long long* __restrict__ mx,
                             int* __restrict__ E) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= R) return;
  const int e = oz_exponent(__longlong_as_double((long long)mx[i]));
  E[i] = e == OZ_ZERO_EXP ? e : e + 1;
}

// Left dd factor -> residue planes [L][Mp][Kp].  Block: 32 rows x 64 k;
// lane = row, warp q takes k0 + 8q .. k0 + 8q + 7 (coalesced loads across
// the warp); the plane tiles go out through shared memory (TileStore).
template <int NL>
__global__ void __launch_bounds__(256)
dd_split_left(int M, int K, int Mp, int Kp, const double* __restrict__ A, long lda, int L, int w,
              const int* __restrict__ E, uint16_t* __restrict__ planes) {
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const int i = blockIdx.y * 32 + lane;
  const int k0 = blockIdx.x * 64 + wq * 8;
  const int Ei = i < M ? E[i] : OZ_ZERO_EXP;
  unsigned __int128 ua[8];
  unsigned negm = 0;
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const int k = k0 + t;
    double hi = 0.0, lo = 0.0;
    if (i < M && k < K) {
      const double2 e = *reinterpret_cast<const double2*>(A + 2 * (i + (long)k * lda));
      if (isfinite(e.x) && isfinite(e.y)) {
        hi = e.x;
        lo = e.y;
      }
    }
    const __int128 a = dd_int(hi, lo, Ei, w);
    ua[t] = (unsigned __int128)(a < 0 ? -a : a);
    if (a < 0) negm |= 1u << t;
  }
  __shared__ uint4 tile_smem[2][32][9];
  TileStore ts{tile_smem, 0};
  const size_t tile0 = (size_t)(blockIdx.y * 32) * Kp + blockIdx.x * 64;
  const size_t pstride = (size_t)Mp * Kp;
  float hl[8][NL];
#pragma unroll
  for (int t = 0; t < 8; ++t) limbs12<NL>(ua[t], (negm >> t) & 1u, hl[t]);
#pragma unroll
  for (int l = 0; l < OZ_MAX_MODULI; ++l) {
    if (l >= L) break;
    uint32_t h[4];
#pragma unroll
    for (int t = 0; t < 8; t += 2)
      h[t / 2] = res_pair<NL>(hl[t], hl[t + 1], l);
    ts.put(make_uint4(h[0], h[1], h[2], h[3]), planes + l * pstride + tile0, Kp);
  }
}

// Right dd factor, pass 1: one warp per column (8 per block), the column
// maximum of |hi| (warp reduction) and its exponent; padding columns get
// the zero exponent.
__global__ void __launch_bounds__(256)
dd_colmax(int K, int N, int Np, const double* __restrict__ B, long ldb, int* __restrict__ F,
          int* __restrict__ flag) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (j >= Np) return;  // whole warps only
  unsigned long long am = 0;
  bool bad = false;
  if (j < N) {
    const double* bcol = B + 2 * (long)j * ldb;
    for (int k = lane; k < K; k += 32) {
      const double2 e = *reinterpret_cast<const double2*>(bcol + 2 * k);
      if (sw_finite(e.x) && sw_finite(e.y))
        am = max(am, dbits(oz_abs(e.x)));
      else
        bad = true;
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flag, 1);
  am = warp_max_u64(am);
  int Fj = oz_exponent(__longlong_as_double((long long)am));
  if (Fj != OZ_ZERO_EXP) Fj += 1;
  if (lane == 0) F[j] = j < N ? Fj : OZ_ZERO_EXP;
}

// Right dd factor, pass 2 -> residue planes [L][Np][Kp].  Block: 8 columns x
// 256 k; warp q takes column 8 bx.y + q, lane t the 8 consecutive k of
// 256 bx.x + 8 t .. + 7 (each warp reads 4 KB of its column contiguously and
// writes 512 contiguous bytes per plane).
template <int NL>
__global__ void __launch_bounds__(256)
dd_split_right(int K, int N, int Kp, int Np, const double* __restrict__ B, long ldb, int L, int w,
               const int* __restrict__ F, uint16_t* __restrict__ planes) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int k0 = blockIdx.x * 256 + 8 * lane;
  if (j >= Np || k0 >= Kp) return;
  const int Fj = F[j];
  const double* bcol = B + 2 * (long)j * ldb;
  float hl[8][NL];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const int k = k0 + t;
    double hi = 0.0, lo = 0.0;
    if (j < N && k < K) {
      const double2 e = *reinterpret_cast<const double2*>(bcol + 2 * k);
      if (sw_finite(e.x) && sw_finite(e.y)) {
        hi = e.x;
        lo = e.y;
      }
    }
    const __int128 b = dd_int(hi, lo, Fj, w);
    limbs12<NL>((unsigned __int128)(b < 0 ? -b : b), b < 0, hl[t]);
  }
  const size_t pstride = (size_t)Np * Kp, off = (size_t)j * Kp + k0;
#pragma unroll
  for (int l = 0; l < OZ_MAX_MODULI; ++l) {
    if (l >= L) break;
    uint32_t h[4];
#pragma unroll
    for (int t = 0; t < 8; t += 2)
      h[t / 2] = res_pair<NL>(hl[t], hl[t + 1], l);
    *reinterpret_cast<uint4*>(planes + l * pstride + off) = make_uint4(h[0], h[1], h[2], h[3]);
  }
}

int dd_prepare(int M, int N, int K, int Mp, int Np, int Kp, int L, int w, const double* A,
               long lda, const double* B, long ldb, unsigned long long* rowmax, int* E, int* F,
               uint16_t* planesA, uint16_t* planesB, int* flag, cudaStream_t st) {
  VCPCU_CUDA_TRY(cudaMemsetAsync(rowmax, 0, sizeof(unsigned long long) * (size_t)Mp, st));
  VCPCU_CUDA_TRY(cudaMemsetAsync(flag, 0, 4 * sizeof(int), st));
  if (M > 0 && K > 0) {
    const int cpb = 256;
    dim3 g1((M + 31) / 32, (K + cpb - 1) / cpb);
    dd_rowmax<<<g1, 256, 0, st>>>(M, K, A, lda, cpb, rowmax, flag);
    VCPCU_LAUNCH_CHECK("dd_rowmax");
  }
  dd_exponents<<<(Mp + 255) / 256, 256, 0, st>>>(Mp, rowmax, E);
  VCPCU_LAUNCH_CHECK("dd_exponents");
  dim3 g2(Kp / 64, Mp / 32);
  // |A'|, |B'| < 2^(w-1): eight 13-bit limbs up to w = 104, ten 12-bit ones
  // up to w = 120
  if (w <= 104)
    dd_split_left<8><<<g2, 256, 0, st>>>(M, K, Mp, Kp, A, lda, L, w, E, planesA);
  else
    dd_split_left<10><<<g2, 256, 0, st>>>(M, K, Mp, Kp, A, lda, L, w, E, planesA);
  VCPCU_LAUNCH_CHECK("dd_split_left");
  dd_colmax<<<(Np + 7) / 8, 256, 0, st>>>(K, N, Np, B, ldb, F, flag);
  VCPCU_LAUNCH_CHECK("dd_colmax");
  dim3 g3((Kp + 255) / 256, Np / 8);
  if (w <= 104)
    dd_split_right<8><<<g3, 256, 0, st>>>(K, N, Kp, Np, B, ldb, L, w, F, planesB);
  else
    dd_split_right<10><<<g3, 256, 0, st>>>(K, N, Kp, Np, B, ldb, L, w, F, planesB);
  VCPCU_LAUNCH_CHECK("dd_split_right");
  return VCPCU_OK;
}

}  // namespace vcpcu
