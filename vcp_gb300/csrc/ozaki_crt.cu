// ozaki_crt.cu -- reassembly of the CRT (Ozaki-II) form of the midpoint
// product and the final enclosure.
//
// For each entry the slice GEMM left the residues c_l = (A'B')(i,j) mod m_l
// (l < L) of the exact integer product of the w-bit operands
// A' = round(mA 2^(w-E_i)), B' = round(mB 2^(w-F_j)).  Chinese remaindering
// gives X = sum_l c_l Q_l mod M (Q_l = (M/m_l) ((M/m_l)^-1 mod m_l)), taken
// in (-M/4, M/4); since prod m_l > 4 |A'B'|, X = (A'B')(i,j) exactly.  Then
//   mA mB = 2^(E+F-2w) X + ΔA mB + Â ΔB,   |ΔA| <= 2^(E-w-1), |ΔB| <= 2^(F-w-1),
//   |ΔA mB| <= 2^(E-w-1) beta_j,   |Â ΔB| <= 2^(E+F-2w-1) sum_k |A'(i,k)|,
// and the enclosure is [RD(2^(E+F-2w) X) - e, RU(2^(E+F-2w) X) + e] with
// e = RU(RU(trunc) + T(i,j)), T the upper bound of the radius term.
#include "common.cuh"
#include "ozaki.cuh"
#include "ozaki_common.cuh"
#include "swfp.cuh"

namespace vcpcu {

namespace {

struct CrtConst {
  uint32_t Q[16][4];
  uint32_t M[4];
  float invMf;  // 2^64 / M rounded to float: the quotient estimate of the reduction
};

__device__ __forceinline__ double scale_dir2(double x, int e, bool up) {
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

// x * 2^e rounded up (up) or down: the exponent field is moved on the
// integer pipe when x and the result are normal (then the product is exact
// and equals scale_dir2's); otherwise scale_dir2.
__device__ __forceinline__ double scale_pow2(double x, int e, bool up) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7ff);
  if (be != 0 && be != 0x7ff && be + e >= 1 && be + e <= 2046)
    return __longlong_as_double((long long)(b + ((unsigned long long)(long long)e << 52)));
  if (oz_zero(x)) return x;
  return scale_dir2(x, e, up);
}

// RD and RU of t * 2^e for t > 0 (64 bits) built on the integer pipe: the
// top 53 bits of t are the truncated significand, any lower bit set makes
// RU one unit larger (a carry into the exponent field is the correct
// rounding).  Equal to scale_dir2(__ull2double_rd/ru(t), e) -- which runs
// when the result leaves the normal range.
__device__ __forceinline__ void u64_to_dir(unsigned long long t, int e, double& dn, double& upv) {
  const int lz = __clzll(t);
  const unsigned long long tn = t << lz;
  const int be = 1023 + 63 - lz + e;
  if (be >= 1 && be <= 2046) {
    const unsigned long long d =
        ((unsigned long long)be << 52) + ((tn >> 11) & ((1ULL << 52) - 1));
    dn = __longlong_as_double((long long)d);
    upv = __longlong_as_double((long long)(d + ((tn & 0x7ffULL) ? 1ULL : 0ULL)));
    return;
  }
  dn = scale_dir2(__ull2double_rd(t), e, false);
  upv = scale_dir2(__ull2double_ru(t), e, true);
}

// Directed conversion of (-1)^neg * mag * 2^e (mag: 4 limbs) to double.
// Limbs are picked by unrolled selects (no dynamically indexed array, which
// would live in local memory).
__device__ __forceinline__ void big_to_dir(const uint32_t (&mag)[4], int neg, int e, double& lo,
                                           double& up) {
  int bl = 0;  // bit length, 0..128
#pragma unroll
  for (int t = 0; t < 4; ++t)
    if (mag[t]) bl = 32 * t + (32 - __clz(mag[t]));
  if (bl == 0) {
    lo = up = 0.0;
    return;
  }
  const int sh = bl > 64 ? bl - 64 : 0;
  const int wq = sh >> 5, bq = sh & 31;
  unsigned long long w0 = 0, w1 = 0, w2 = 0;
  uint32_t below = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (q == wq) w0 = mag[q];
    if (q == wq + 1) w1 = mag[q];
    if (q == wq + 2) w2 = mag[q];
    if (q < wq) below |= mag[q];
  }
  const unsigned long long lo64 = w0 | (w1 << 32);
  unsigned long long t = bq ? ((lo64 >> bq) | (w2 << (64 - bq))) : lo64;
  if (bq) below |= (uint32_t)w0 & ((1u << bq) - 1u);
  if (below) t |= 1ULL;
  double a_dn, a_up;
  u64_to_dir(t, e + sh, a_dn, a_up);
  if (!neg) {
    lo = a_dn;
    up = a_up;
  } else {
    lo = sw_neg(a_up);
    up = sw_neg(a_dn);
  }
}

// Nearest integer of |x| < 2^22 on the FP32 pipe (ties to even).
__device__ __forceinline__ float rint_f(float x) {
  return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f);
}

// u32 -> float rounded to nearest (equal to __uint2float_rn) on the FP32
// pipe: the two 16-bit halves are exact floats, one FMA rounds their sum.
__device__ __forceinline__ float u32_to_f(uint32_t v) {
  const float h = __fsub_rn(__uint_as_float(0x4B000000u | (v >> 16)), 8388608.0f);
  const float l = __fsub_rn(__uint_as_float(0x4B000000u | (v & 0xffffu)), 8388608.0f);
  return __fmaf_rn(h, 65536.0f, l);
}

// Exact X = (A'B')(i, j) from its residues (see the file comment); returns
// the magnitude in mag[4] and the sign.
// c[l] = 0 and Q_l = 0 for l >= L.  S = sum_l c_l Q_l < 2^12 M is formed
// exactly in five 32-bit limbs; the plan keeps |X| <= K 2^(2w-2) < M / 4
// (prod m_l > K 2^(2w)), so S / M lies within 1/4 of the integer q with
// S = q M + X, and the fp32 estimate of S / M (relative error below 2^-20,
// absolute below 2^-8) rounds to exactly that q: X = S - q M in one
// multiply-subtract, already centred, with no correction step.
__device__ __forceinline__ int crt_value(const uint32_t (&c)[16], const uint32_t (&Q)[16][4],
                                         const uint32_t (&Mm)[4], float invMf,
                                         uint32_t (&mag)[4]) {
  unsigned long long s[4] = {0, 0, 0, 0};
#pragma unroll
  for (int l = 0; l < 16; ++l) {
#pragma unroll
    for (int t = 0; t < 4; ++t) s[t] += (unsigned long long)c[l] * Q[l][t];
  }
  uint32_t r[5];
  unsigned long long carry = 0;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const unsigned long long v = s[t] + carry;
    r[t] = (uint32_t)v;
    carry = v >> 32;
  }
  r[4] = (uint32_t)carry;
  const float Sf = u32_to_f(r[4]) * 0x1p64f + u32_to_f(r[3]) * 0x1p32f + u32_to_f(r[2]) +
                   u32_to_f(r[1]) * 0x1p-32f + u32_to_f(r[0]) * 0x1p-64f;
  const unsigned int q = (unsigned int)rint_f(Sf * invMf);  // nearest integer to S / M
  unsigned long long c2 = 0, borrow = 0;
#pragma unroll
  for (int t = 0; t < 5; ++t) {  // r = S - q M in five-limb two's complement
    const unsigned long long v = (t < 4 ? (unsigned long long)q * Mm[t] : 0ULL) + c2;
    c2 = v >> 32;
    const unsigned long long d = (unsigned long long)r[t] - (uint32_t)v - borrow;
    r[t] = (uint32_t)d;
    borrow = (d >> 63) & 1ULL;
  }
  const int neg = (int)(r[4] >> 31);  // |X| < 2^125: the top limb is 0 or all ones
  if (neg) {  // magnitude = -r
    unsigned long long cy = 1;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const unsigned long long v = (unsigned long long)(~r[t]) + cy;
      mag[t] = (uint32_t)v;
      cy = v >> 32;
    }
  } else {
#pragma unroll
    for (int t = 0; t < 4; ++t) mag[t] = r[t];
  }
  return neg;
}

// The radius sums of both products for 4 consecutive rows (e0 = j Mp + i0):
// one fp32 fold per product (slot 0 and slot nslot = 1), the slice GEMM
// epilogue's upward sum of every chunk weighted by its digit pair -- an
// upper bound of the exact integer W of the product.
__device__ __forceinline__ void rad_folds(const int32_t* __restrict__ P, size_t plane,
                                          size_t e0, const OzRadConst& rc, float (&S1)[4],
                                          float (&S2)[4]) {
  const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float4 v1 = rc.run1 ? *reinterpret_cast<const float4*>(P + e0) : z;
  const float4 v2 =
      rc.run2 ? *reinterpret_cast<const float4*>(P + (size_t)rc.nslot * plane + e0) : z;
  S1[0] = v1.x;
  S1[1] = v1.y;
  S1[2] = v1.z;
  S1[3] = v1.w;
  S2[0] = v2.x;
  S2[1] = v2.y;
  S2[2] = v2.z;
  S2[3] = v2.w;
}

// RU(sqrt(RU(Q))) scale for a sum Q of squared low radius digits (0 for
// Q = 0; scale a power of two, so the product is exact).
__device__ __forceinline__ float lowpair_root(unsigned long long Q, float scale) {
  return Q ? __fmul_rn(__fsqrt_ru(__ull2float_ru(Q)), scale) : 0.0f;
}

// RU(RU(S + R) + b) 2^ex, 0 for a zero row or column.  S + R >= the exact
// W + R of the pairs that ran; b >= the left-out low x low pair (in the units
// of W: sum_k lo_A lo_B 2^-8 <= sqrt(sum lo_A^2) sqrt(sum lo_B^2) 2^-8,
// Cauchy-Schwarz), 0 when every pair ran.  The sum is >= 0 (the digits of
// both radius factors are upward, so every product of their reconstructions
// is non-negative) and is 0 or at least 2^-16: a normal float, whose double
// is built on the integer pipe.
__device__ __forceinline__ double rad_term(float S, bool zero, int ex, int R, float b) {
  if (zero) return 0.0;
  float s = R ? __fadd_ru(S, (float)R) : S;
  s = __fadd_ru(s, b);
  if (!(s > 0.0f)) return 0.0;
  const unsigned u = __float_as_uint(s);
  const double d = __longlong_as_double((long long)(((unsigned long long)((u >> 23) + 896) << 52) |
                                                    ((unsigned long long)(u & 0x7fffffu) << 29)));
  return scale_pow2(d, ex, true);
}

// T = RU(RU((|mA| + rA) rB) + RU(rA |mB|)) at (i, j), the products that ran;
// l1, l2 the bounds of their left-out pairs.
__device__ __forceinline__ double rad_T(float S1, float S2, int Ep, int Er, int Fm, int Fr,
                                        const OzRadConst& rc, float l1, float l2) {
  const double b1 = rc.run1 ? rad_term(S1, Ep == OZ_ZERO_EXP || Fr == OZ_ZERO_EXP,
                                       Ep + Fr - 8 * rc.t_ref, rc.R, l1)
                            : 0.0;
  if (!rc.run2) return b1;
  const double b2 =
      rad_term(S2, Er == OZ_ZERO_EXP || Fm == OZ_ZERO_EXP, Er + Fm - 8 * rc.t_ref, rc.R, l2);
  return rc.run1 ? __dadd_ru(b1, b2) : b2;
}

// Slice form: T (ld Mp) from the folds, before the midpoint product.
__global__ void __launch_bounds__(256)
oz_radius_T_kernel(int M, int N, int Mp, size_t plane, const int32_t* __restrict__ P,
                   const int* __restrict__ E3, const int* __restrict__ F2,
                   double* __restrict__ T, const __grid_constant__ OzRadConst rc) {
  const int Mq = (M + 3) >> 2;
  const long total = (long)Mq * N;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int i0 = 4 * (int)(idx % Mq), j = (int)(idx / Mq);
    const size_t e0 = (size_t)j * Mp + i0;
    float W1[4], W2[4];
    rad_folds(P, plane, e0, rc, W1, W2);
    const int Fm = F2[2 * j], Fr = F2[2 * j + 1];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u;
      if (i >= M) break;
      T[e0 + u] = rad_T(W1[u], W2[u], E3[3 * i + 1], E3[3 * i + 2], Fm, Fr, rc, 0.0f, 0.0f);
    }
  }
}

// Per-row data of 4 consecutive rows: the exponents, sA = RU(sum_k
// |A'(i,k)|) (asum_hi 2^32 + asum_lo, exact below 2^96) and the 2^-8-scaled
// roots of the low radius digits' squares of P and rA, computed once per
// thread and reused for every column it assembles.
struct QuadRows {
  int E[4], Ep[4], Er[4];
  double sA[4];
  float qp[4], qr[4];
};

__device__ __forceinline__ void quad_rows(int i0, int M, const int* __restrict__ E3,
                                          const unsigned long long* __restrict__ asum,
                                          QuadRows& r) {
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = i0 + u;
    r.E[u] = r.Ep[u] = r.Er[u] = OZ_ZERO_EXP;
    r.sA[u] = 0.0;
    r.qp[u] = r.qr[u] = 0.0f;
    if (i >= M) continue;
    r.E[u] = E3[3 * i];
    r.Ep[u] = E3[3 * i + 1];
    r.Er[u] = E3[3 * i + 2];
    r.qp[u] = lowpair_root(asum[4 * i + 2], 0x1p-8f);
    r.qr[u] = lowpair_root(asum[4 * i + 3], 0x1p-8f);
    const unsigned long long ah = asum[4 * i + 0], al = asum[4 * i + 1];
    const unsigned __int128 sx = ((unsigned __int128)ah << 32) + al;
    if (sx) {
      double sAdn;
      const unsigned long long hi64 = (unsigned long long)(sx >> 64);
      if (hi64 == 0) {
        u64_to_dir((unsigned long long)sx, 0, sAdn, r.sA[u]);
      } else {
        const int sh = 64 - __clzll(hi64);
        unsigned long long t = (unsigned long long)(sx >> sh);
        if ((unsigned long long)sx & ((1ULL << sh) - 1)) t |= 1ULL;
        u64_to_dir(t, sh, sAdn, r.sA[u]);
      }
    }
  }
}

// The 4 entries (i0 .. i0+3, j): the residue planes are read 4 bytes at a
// time, the radius folds 16 bytes, C written as 4 consecutive pairs.  Only
// the final error sum and the two outward roundings use the FP64 pipe on the
// common path.  res and P point at row / column 0 of this product; plane =
// Np Mp of its layout; Fj, Frj the column's exponents, bj its beta, qj its
// sums of squared low radius digits (of rB and |mB|).
__device__ __forceinline__ void assemble_quad_col(
    const QuadRows& rw, int i0, int j, int M, int Mp, int L, int w,
    const uint8_t* __restrict__ res, size_t plane, int Fj, int Frj, double bj,
    const unsigned long long* __restrict__ qj, const int32_t* __restrict__ P,
    double* __restrict__ C, long ldc, bool nonfinite, const uint32_t (&Q)[16][4],
    const uint32_t (&Mm)[4], float invMf, const OzRadConst& rc) {
  const size_t e0 = (size_t)j * Mp + i0;
  uint32_t pk[16];
#pragma unroll
  for (int l = 0; l < 16; ++l)
    pk[l] = l < L ? *reinterpret_cast<const uint32_t*>(res + (size_t)l * plane + e0) : 0u;
  float W1[4], W2[4];
  rad_folds(P, plane, e0, rc, W1, W2);
  const float qb1 = rc.lowb ? lowpair_root(qj[0], 1.0f) : 0.0f;
  const float qb2 = rc.lowb ? lowpair_root(qj[1], 1.0f) : 0.0f;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = i0 + u;
    if (i >= M) break;
    const int Ei = rw.E[u];
    double lo = 0.0, up = 0.0, tr = 0.0;
    if (Ei != OZ_ZERO_EXP && Fj != OZ_ZERO_EXP) {
      uint32_t c[16], mag[4];
#pragma unroll
      for (int l = 0; l < 16; ++l) c[l] = (pk[l] >> (8 * u)) & 0xffu;
      const int neg = crt_value(c, Q, Mm, invMf, mag);
      big_to_dir(mag, neg, Ei + Fj - 2 * w, lo, up);
      const double t1 = scale_pow2(bj, Ei - w - 1, true);
      const double t2 = scale_pow2(rw.sA[u], Ei + Fj - 2 * w - 1, true);
      tr = __dadd_ru(t1, t2);
    }
    const double Tu = rad_T(W1[u], W2[u], rw.Ep[u], rw.Er[u], Fj, Frj, rc,
                            __fmul_ru(rw.qp[u], qb1), __fmul_ru(rw.qr[u], qb2));
    const double err = __dadd_ru(tr, Tu);
    double clo = __dsub_rd(lo, err), cup = __dadd_ru(up, err);
    if (nonfinite) clo = cup = __longlong_as_double(0x7ff8000000000000LL);
    double* cp = C + 2 * ((size_t)i + (size_t)j * ldc);  // C may be only 8-byte aligned
    cp[0] = clo;
    cp[1] = cup;
  }
}

// Thread = 4 consecutive rows of about 8 columns; blockIdx.y strides over the
// columns (no 64-bit index division).  At most 80 registers: three blocks per
// SM (measured at n = 8192: 1.88 ms; 2.10 ms at the unbounded 94 registers).
__global__ void __launch_bounds__(256, 3)
oz_crt_assemble_kernel(int M, int N, int Mp, int L, int w, const uint8_t* __restrict__ res,
                       size_t plane, const int* __restrict__ E3, const int* __restrict__ F2,
                       const unsigned long long* __restrict__ asum,
                       const unsigned long long* __restrict__ bsum,
                       const double* __restrict__ beta, const int32_t* __restrict__ P,
                       double* __restrict__ C, long ldc, const int* __restrict__ flag,
                       const __grid_constant__ CrtConst cc, const __grid_constant__ OzRadConst rc) {
  const bool nonfinite = flag[0] != 0 || flag[1] != 0;
  const int Mq = (M + 3) >> 2;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Mq) return;
  QuadRows rw;
  quad_rows(4 * q, M, E3, asum, rw);
  for (int j = blockIdx.y; j < N; j += gridDim.y)
    assemble_quad_col(rw, 4 * q, j, M, Mp, L, w, res, plane, F2[2 * j], F2[2 * j + 1], beta[j],
                      bsum + 4 * (size_t)j + 2, P, C, ldc, nonfinite, cc.Q, cc.M, cc.invMf, rc);
}

// Grouped reassembly.  The problems of a bucket share one CRT plan (the
// bucket is keyed by padded K, modulus count and operand width), so the
// basis comes in the launch parameters as for one product.  A thread takes 4
// consecutive rows of one problem and the columns cg, cg + NG, cg + 2 NG, ...
// (NG = ceil(n / 8) column groups): its rows' exponents and sums are set up
// once for about 8 columns, and consecutive threads take consecutive row
// quads (coalesced residue and fold reads).  A block finds its problem with
// one load (prob_asm), stamps the problem's end and merges its status words
// into the sticky status.  A device-wait timeout of the slice
// GEMM (flag[1] of problem 0) poisons every output of the bucket.  117
// registers: two blocks per SM (the problem's pointers and sizes stay in
// registers where one product has them in the launch parameters; at 80
// registers they spill).
__global__ void __launch_bounds__(256, 2)
oz_crt_assemble_g(const __grid_constant__ OzGBucket b, const __grid_constant__ CrtConst cc,
                  const __grid_constant__ OzRadConst rc, int* __restrict__ status) {
  const int p = b.prob_asm[blockIdx.x];
  const OzGProb& q = b.probs[p];
  const int m = q.m, n = q.n;
  const int Mq = (m + 3) >> 2;
  const int NG = (n + 7) >> 3;
  const long u = (long)(blockIdx.x - b.blk_asm[p]) * blockDim.x + threadIdx.x;
  const int f0 = b.flag[4 * p], f1 = b.flag[4 * p + 1];
  if (u < (long)Mq * NG) {
    const bool nonfinite = f0 != 0 || b.flag[1] != 0;
    const int qd = (int)(u % Mq), cg = (int)(u / Mq);
    const int* E3 = b.E3 + 3 * (size_t)q.rowoff;
    const unsigned long long* asum = b.asum + 4 * (size_t)q.rowoff;
    const unsigned long long* bsum = b.bsum + 4 * (size_t)q.coloff;
    const int* F2 = b.F2 + 2 * (size_t)q.coloff;
    const double* beta = b.beta + q.coloff;
    const uint8_t* res = b.res + q.res_off;
    const int32_t* P = b.P + q.P_off;
    const size_t plane = (size_t)q.Np * q.Mp;
    QuadRows rw;
    quad_rows(4 * qd, m, E3, asum, rw);
    for (int j = cg; j < n; j += NG)
      assemble_quad_col(rw, 4 * qd, j, m, q.Mp, q.L, q.w, res, plane, F2[2 * j], F2[2 * j + 1],
                        beta[j], bsum + 4 * (size_t)j + 2, P, q.C, q.ldc, nonfinite, cc.Q, cc.M,
                        cc.invMf, rc);
  }
  if (threadIdx.x == 0 && (f0 | f1)) atomicOr(status, (f0 ? 1 : 0) | (f1 ? 2 : 0));
  if (b.t_last) {
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      atomicMax(&b.t_last[q.orig], t);
    }
  }
}

}  // namespace

namespace {
// The CRT basis of a plan's L moduli (Q_l = 0 past L), M and 2^64 / M.
CrtConst crt_const(const OzPlan& plan) {
  CrtConst cc;
  memset(&cc, 0, sizeof(cc));
  for (int l = 0; l < plan.pb.L; ++l)
    for (int t = 0; t < 4; ++t) cc.Q[l][t] = plan.Q[l][t];
  for (int t = 0; t < 4; ++t) cc.M[t] = plan.Mlimb[t];
  const double Md = (double)cc.M[3] * 0x1p96 + (double)cc.M[2] * 0x1p64 +
                    (double)cc.M[1] * 0x1p32 + (double)cc.M[0];
  cc.invMf = (float)(0x1p64 / Md);
  return cc;
}
}  // namespace

int oz_crt_assemble(const OzPlan& plan, const OzWorkspace& ws, double* C, long ldc,
                    cudaStream_t st) {
  const OzProblem& pb = plan.pb;
  const CrtConst cc = crt_const(plan);
  if (pb.M <= 0 || pb.N <= 0) return VCPCU_OK;
  const int Mq = (pb.M + 3) / 4;
  // about 8 columns per thread: its rows' exponents and sums are set up once
  const int gy = (pb.N + 7) / 8;
  // 128-thread blocks: a row count that is not a multiple of 1024 leaves at
  // most 127 idle threads per column group (the blocks of a host-pointer
  // product have 768 - 1536 rows)
  dim3 grid((Mq + 127) / 128, gy < 65535 ? gy : 65535);
  oz_crt_assemble_kernel<<<grid, 128, 0, st>>>(
      pb.M, pb.N, pb.Mp, pb.L, pb.w, ws.res, (size_t)pb.Np * pb.Mp, ws.E3, ws.F2, ws.asum,
      ws.bsum, ws.beta, ws.P, C, ldc, ws.flag, cc, oz_rad_const(plan));
  VCPCU_LAUNCH_CHECK("oz_crt_assemble_kernel");
  return VCPCU_OK;
}

int oz_gassemble(const OzGBucket& b, const OzPlan& shape, const OzRadConst& rc, int nblk,
                 cudaStream_t st) {
  if (nblk <= 0) return VCPCU_OK;
  int* status = oz_status_ptr();
  if (!status) {
    set_error("igemm_batched: no device address of the status word");
    return VCPCU_ERR_CUDA;
  }
  oz_crt_assemble_g<<<nblk, 256, 0, st>>>(b, crt_const(shape), rc, status);
  VCPCU_LAUNCH_CHECK("oz_crt_assemble_g");
  return VCPCU_OK;
}

int oz_radius_T(const OzPlan& plan, const OzWorkspace& ws, cudaStream_t st) {
  const OzProblem& pb = plan.pb;
  const long total = (long)((pb.M + 3) / 4) * pb.N;
  long blocks = (total + 255) / 256;
  if (blocks > 152L * 64) blocks = 152L * 64;
  if (blocks < 1) blocks = 1;
  oz_radius_T_kernel<<<(int)blocks, 256, 0, st>>>(pb.M, pb.N, pb.Mp, (size_t)pb.Np * pb.Mp, ws.P,
                                                  ws.E3, ws.F2, ws.T, oz_rad_const(plan));
  VCPCU_LAUNCH_CHECK("oz_radius_T_kernel");
  return VCPCU_OK;
}

}  // namespace vcpcu
