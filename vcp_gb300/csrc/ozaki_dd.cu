// ozaki_dd.cu -- double-double GEMM (the vcp::pddcuda policy, pddblas
// semantics: vcp/pddblas.hpp:318-409) on the tensor cores.
//
// pddblas splits each dd operand into double slices, multiplies every slice
// pair with dgemm and accumulates the exact products in dd
// (pddblas_assist::split_row / split_col / ozaki_acc, vcp/pddblas.hpp:82-193).
// Here each dd entry hi + lo is scaled per row (A) / column (B) to a w-bit
// integer (w = 8 * slices, default 112 bits), the integer product A'B' is
// formed exactly from its residues modulo L <= 32 pairwise-coprime moduli
// <= 256 (one bf16 tensor-core GEMM per modulus, exact fp32 chunks, int32
// folds), recovered by Chinese remaindering in 256-bit arithmetic, and
// rounded to a dd midpoint C = chi + clo.  A rigorous upward-rounded bound
//   |A B - C| <= K 2^(E+F-w) (1 + 2^-40) + ulp-level conversion error
// is returned alongside (Cerr).  Inputs and outputs use kv::dd layout:
// pairs {a1, a2} of doubles, column-major.
#include "common.cuh"
#include "ozaki.cuh"
#include "ozaki_common.cuh"
#include "swfp.cuh"

#include <cmath>
#include <cstring>

namespace vcpcu {

int dd_prepare(int M, int N, int K, int Mp, int Np, int Kp, int L, int w, const double* A,
               long lda, const double* B, long ldb, unsigned long long* rowmax, int* E, int* F,
               uint16_t* planesA, uint16_t* planesB, int* flag, cudaStream_t st);

namespace {

constexpr int DDL = 8;  // 32-bit limbs of the CRT modulus (M < 2^256)

struct DdCrt {
  uint32_t Q[OZ_MAX_MODULI][DDL];
  uint32_t M[DDL];
  // FP32 quotient estimate of r / M: r ~ sum_t r[t] pw[t] 2^e0 and
  // M ~ 2^e0 / invMf with e0 = 32 (topM - 1), topM the top nonzero limb of M
  // (pw[t] = 0 outside topM - 1 .. topM + 1).
  float pw[DDL + 1];
  float invMf;
};

// ---- host: basis of the CRT in 256-bit arithmetic -------------------------
void big_mul_small(uint32_t* a, uint32_t s) {
  unsigned long long c = 0;
  for (int t = 0; t < DDL; ++t) {
    const unsigned long long v = (unsigned long long)a[t] * s + c;
    a[t] = (uint32_t)v;
    c = v >> 32;
  }
}
uint32_t big_div_small(const uint32_t* a, uint32_t s, uint32_t* q) {
  unsigned long long r = 0;
  for (int t = DDL - 1; t >= 0; --t) {
    const unsigned long long v = (r << 32) | a[t];
    q[t] = (uint32_t)(v / s);
    r = v % s;
  }
  return (uint32_t)r;
}

int dd_crt_setup(int K, int* w, int* L, DdCrt* c) {
  const int Keff = K > 1 ? K : 1;
  for (;;) {
    const double need = (2.0 * *w - 1.0) + std::log2((double)Keff) + 0.01;
    double bits = 0.0;
    int l = 0;
    while (l < OZ_MAX_MODULI && bits <= need) bits += std::log2((double)OZ_MODULI[l++]);
    if (bits > need) {
      *L = l;
      break;
    }
    --*w;
  }
  memset(c, 0, sizeof(*c));
  c->M[0] = 1;
  for (int l = 0; l < *L; ++l) big_mul_small(c->M, (uint32_t)OZ_MODULI[l]);
  for (int l = 0; l < *L; ++l) {
    const uint32_t m = (uint32_t)OZ_MODULI[l];
    uint32_t Ml[DDL];
    big_div_small(c->M, m, Ml);
    uint32_t tmp[DDL];
    const uint32_t r = big_div_small(Ml, m, tmp);
    uint32_t inv = 0;
    for (uint32_t x = 1; x < m; ++x)
      if ((r * x) % m == 1) {
        inv = x;
        break;
      }
    memcpy(c->Q[l], Ml, sizeof(Ml));
    big_mul_small(c->Q[l], inv);  // (M/m_l) * inv < M
  }
  int topM = DDL - 1;
  while (topM > 0 && c->M[topM] == 0) --topM;
  const int e0 = 32 * (topM - 1);
  double Ms = 0.0;
  for (int t = (topM > 0 ? topM - 1 : 0); t <= topM; ++t)
    Ms += std::ldexp((double)c->M[t], 32 * t - e0);
  for (int t = 0; t <= DDL; ++t)
    c->pw[t] = (t >= topM - 1 && t <= topM + 1) ? (float)std::ldexp(1.0, 32 * t - e0) : 0.0f;
  c->invMf = (float)(1.0 / Ms);
  return 0;
}

// ---- device ---------------------------------------------------------------
// All the reassembly arithmetic runs on the integer and FP32 pipes; the few
// FP64 instructions left sit on paths taken only near the ends of the
// double range.
__device__ __forceinline__ double bits_to_d(unsigned long long b) {
  return __longlong_as_double((long long)b);
}
__device__ __forceinline__ unsigned long long d_to_bits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// Highest set bit + 1 of a DDL-limb magnitude (0 for zero).
__device__ __forceinline__ int bitlen(const uint32_t (&mag)[DDL]) {
  int bl = 0;
#pragma unroll
  for (int t = 0; t < DDL; ++t)
    if (mag[t]) bl = 32 * t + (32 - __clz(mag[t]));
  return bl;
}

// The top 64 bits of mag (bit length bl > 0) with a sticky bit for anything
// below, and the shift: mag ~ T 2^sh.  Also the exact top bits without the
// sticky bit (Tx) and whether the remainder below them is nonzero.
__device__ __forceinline__ unsigned long long top64(const uint32_t (&mag)[DDL], int bl, int& sh,
                                                    unsigned long long& Tx) {
  sh = bl > 64 ? bl - 64 : 0;
  const int wq = sh >> 5, bq = sh & 31;
  unsigned long long w0 = 0, w1 = 0, w2 = 0;
  uint32_t below = 0;
#pragma unroll
  for (int q = 0; q < DDL; ++q) {
    const uint32_t v = mag[q];
    if (q == wq) w0 = v;
    if (q == wq + 1) w1 = v;
    if (q == wq + 2) w2 = v;
    if (q < wq) below |= v;
  }
  const unsigned long long lo64 = w0 | (w1 << 32);
  const unsigned long long t = bq ? ((lo64 >> bq) | (w2 << (64 - bq))) : lo64;
  if (bq) below |= (uint32_t)w0 & ((1u << bq) - 1u);
  Tx = t;
  return below ? (t | 1ULL) : t;
}

// RN of an integer t > 0 to 53 bits: significand Mh in [2^52, 2^53) and
// shift g with RN(t) = Mh 2^g.
__device__ __forceinline__ unsigned long long u64_rn(unsigned long long t, int& g) {
  const int b = 64 - __clzll(t);
  if (b <= 53) {
    g = b - 53;
    return t << (53 - b);
  }
  const int s = b - 53;
  unsigned long long Mh = t >> s;
  const unsigned long long rem = t & ((1ULL << s) - 1), half = 1ULL << (s - 1);
  if (rem > half || (rem == half && (Mh & 1ULL))) ++Mh;
  g = s;
  if (Mh >> 53) {
    Mh >>= 1;
    ++g;
  }
  return Mh;
}

// The double Mh 2^ex (Mh in [2^52, 2^53), biased exponent known in range).
__device__ __forceinline__ double exp_add(unsigned long long Mh, int ex) {
  return bits_to_d(((unsigned long long)(ex + 52 + 1023) << 52) | (Mh & ((1ULL << 52) - 1)));
}

// RU(x 2^e) for x > 0 through the range-safe FP64 steps.
__device__ double scale_ru_slow(double x, int e) {
  while (e > 1023) {
    x = __dmul_ru(x, 0x1p1023);
    e -= 1023;
  }
  while (e < -1022) {
    x = __dmul_ru(x, 0x1p-1022);
    e += 1022;
  }
  return __dmul_ru(x, __longlong_as_double((long long)(e + 1023) << 52));
}

__global__ void __launch_bounds__(256)
dd_crt_assemble_kernel(int M, int N, int K, int Mp, int L, int w, const uint8_t* __restrict__ res,
                       size_t plane, const int* __restrict__ E, const int* __restrict__ F,
                       double* __restrict__ C, long ldc, double* __restrict__ Cerr, long lde,
                       const int* __restrict__ flag, const __grid_constant__ DdCrt cc) {
  const bool bad = flag[0] != 0 || flag[1] != 0;
  // truncation of the operands to w-bit integers: K 2^(E+F-w) (1 + 2^-40)
  const double kf = __dmul_ru((double)(K > 0 ? K : 0), 1.0 + 0x1p-40);
  const unsigned long long kfb = d_to_bits(kf);
  const int kfe = (int)(kfb >> 52);
  for (int j = blockIdx.y; j < N; j += gridDim.y) {
    const int Fj = F[j];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
      const int Ei = E[i];
      double hi = 0.0, lo = 0.0, err = 0.0;
      if (Ei != OZ_ZERO_EXP && Fj != OZ_ZERO_EXP) {
        const size_t e = (size_t)j * Mp + i;
        unsigned long long s[DDL];
#pragma unroll
        for (int t = 0; t < DDL; ++t) s[t] = 0;
#pragma unroll 4
        for (int l = 0; l < L; ++l) {
          const unsigned long long c = res[(size_t)l * plane + e];
#pragma unroll
          for (int t = 0; t < DDL; ++t) s[t] += c * cc.Q[l][t];
        }
        uint32_t r[DDL + 1];
        unsigned long long carry = 0;
#pragma unroll
        for (int t = 0; t < DDL; ++t) {
          const unsigned long long v = s[t] + carry;
          r[t] = (uint32_t)v;
          carry = v >> 32;
        }
        r[DDL] = (uint32_t)carry;
        // q ~ r / M (r < 2^13 M: q is off by at most one), then r -= q M
        float Rf = 0.0f;
#pragma unroll
        for (int t = DDL; t >= 0; --t) Rf = __fmaf_rn(__uint2float_rn(r[t]), cc.pw[t], Rf);
        const unsigned int q = __float2uint_rd(fmaxf(__fmul_rn(Rf, cc.invMf), 0.0f));
        {
          unsigned long long c2 = 0, borrow = 0;
#pragma unroll
          for (int t = 0; t <= DDL; ++t) {
            const unsigned long long mt = t < DDL ? cc.M[t] : 0u;
            const unsigned long long v = (unsigned long long)q * mt + c2;
            c2 = v >> 32;
            const unsigned long long d = (unsigned long long)r[t] - (uint32_t)v - borrow;
            r[t] = (uint32_t)d;
            borrow = (d >> 63) & 1ULL;
          }
          for (int it = 0; it < 4 && (r[DDL] >> 31); ++it) {  // negative: add M
            unsigned long long cy = 0;
#pragma unroll
            for (int t = 0; t <= DDL; ++t) {
              const unsigned long long v =
                  (unsigned long long)r[t] + (t < DDL ? cc.M[t] : 0u) + cy;
              r[t] = (uint32_t)v;
              cy = v >> 32;
            }
          }
          for (int it = 0; it < 4; ++it) {  // r >= M: subtract
            unsigned long long b = 0;
            uint32_t d[DDL + 1];
#pragma unroll
            for (int t = 0; t <= DDL; ++t) {
              const unsigned long long v =
                  (unsigned long long)r[t] - (t < DDL ? cc.M[t] : 0u) - b;
              d[t] = (uint32_t)v;
              b = (v >> 63) & 1ULL;
            }
            if (b) break;  // r < M
#pragma unroll
            for (int t = 0; t <= DDL; ++t) r[t] = d[t];
          }
        }
        // centre: X = r (2r < M) or r - M
        uint32_t mag[DDL];
        int neg = 0;
        {
          unsigned long long b = 0;
          uint32_t d[DDL];
#pragma unroll
          for (int t = 0; t < DDL; ++t) {  // d = M - r; 2r >= M  <=>  r >= M - r
            const unsigned long long v = (unsigned long long)cc.M[t] - r[t] - b;
            d[t] = (uint32_t)v;
            b = (v >> 63) & 1ULL;
          }
          unsigned long long b2 = 0;
#pragma unroll
          for (int t = 0; t < DDL; ++t) {  // r - d: borrow out means r < d
            const unsigned long long v = (unsigned long long)r[t] - d[t] - b2;
            b2 = (v >> 63) & 1ULL;
          }
          neg = b2 == 0;
#pragma unroll
          for (int t = 0; t < DDL; ++t) mag[t] = neg ? d[t] : r[t];
        }
        // dd of mag * 2^ex: hi = RN, lo = RN of the exact remainder
        const int ex = Ei + Fj - 2 * w;
        const int bl = bitlen(mag);
        bool range_ok = true;
        if (bl > 0) {
          int sh;
          unsigned long long Tx;
          const unsigned long long t = top64(mag, bl, sh, Tx);
          int g;
          const unsigned long long Mh = u64_rn(t, g);
          if (ex + sh < -1022 || ex + sh + 64 > 1023) range_ok = false;
          double hval = range_ok ? exp_add(Mh, g + ex + sh) : 0.0;
          // remainder Y = mag - RN(t) 2^sh = D 2^sh + (mag mod 2^sh), with
          // D = Tx - RN(t) (|D| <= 2^10; the u64 difference wraps exactly)
          const long long D = (long long)(Tx - (g >= 0 ? (Mh << g) : (Mh >> -g)));
          const unsigned long long Dm = (unsigned long long)(D < 0 ? -D : D);
          const int wq = sh >> 5, bq = sh & 31;
          // y = |Y| as limbs: Dm 2^sh + low (D >= 0) or Dm 2^sh - low (D < 0)
          uint32_t y[DDL];
          {
            const unsigned long long ds = Dm << bq;  // < 2^42
            unsigned long long b = 0;
#pragma unroll
            for (int q2 = 0; q2 < DDL; ++q2) {
              uint32_t lowq = q2 < wq ? mag[q2] : 0u;
              if (q2 == wq && bq) lowq = mag[q2] & ((1u << bq) - 1u);
              const uint32_t dq = q2 == wq ? (uint32_t)ds : (q2 == wq + 1 ? (uint32_t)(ds >> 32) : 0u);
              if (D >= 0) {
                y[q2] = dq | lowq;  // disjoint bit ranges
              } else {
                const unsigned long long v = (unsigned long long)dq - lowq - b;
                y[q2] = (uint32_t)v;
                b = (v >> 63) & 1ULL;
              }
            }
          }
          const int yneg = (D < 0) != 0;
          double lval = 0.0;
          const int ybl = bitlen(y);
          if (ybl > 0) {
            int ysh;
            unsigned long long yTx;
            const unsigned long long yt = top64(y, ybl, ysh, yTx);
            int yg;
            const unsigned long long yM = u64_rn(yt, yg);
            const int ye = ex + ysh;
            if (ye < -1022 || ye + 64 > 1023)
              range_ok = false;
            else
              lval = exp_add(yM, yg + ye);
            if (yneg) lval = -lval;
          }
          hi = neg ? -hval : hval;
          lo = neg ? -lval : lval;
          // conversion error <= ulp(lo) (<= |lo| 2^-52) + 2^-1074:
          // RU(|lo| 2^-52 + 2^-1074) is the successor of |lo| 2^-52 when
          // that is normal
          const unsigned long long lb = d_to_bits(lval) & 0x7fffffffffffffffULL;
          if ((lb >> 52) >= 53)
            err = bits_to_d(lb - (52ULL << 52) + 1);
          else
            err = __fma_ru(fabs(lo), 0x1p-52, 0x1p-1074);
        }
        const int et = Ei + Fj - w;
        double tr = 0.0;
        if (kf != 0.0) {
          if (kfe + et >= 1 && kfe + et <= 2046)
            tr = bits_to_d(kfb + ((unsigned long long)(long long)et << 52));
          else
            tr = scale_ru_slow(kf, et);
        }
        err = __dadd_ru(err, tr);
        if (!range_ok) err = INFINITY;
      }
      if (bad) hi = lo = err = __longlong_as_double(0x7ff8000000000000LL);
      C[2 * ((size_t)i + (size_t)j * ldc)] = hi;
      C[2 * ((size_t)i + (size_t)j * ldc) + 1] = lo;
      if (Cerr) Cerr[(size_t)i + (size_t)j * lde] = err;
    }
  }
}

size_t al256d(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

int dd_plan_bits(int k, int slices, int* w, int* L) {
  DdCrt c;
  *w = 8 * slices;
  return dd_crt_setup(k, w, L, &c);
}

int ozaki_ddgemm(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                 double* C, long ldc, double* Cerr, long lde, int slices, cudaStream_t s,
                 void* static_scratch, size_t static_bytes) {
  int w = 8 * (slices > 0 ? slices : 14), L = 0;
  DdCrt cc;
  dd_crt_setup(k, &w, &L, &cc);
  OzPlan plan;
  memset(&plan, 0, sizeof(plan));
  OzProblem& pb = plan.pb;
  pb.M = m;
  pb.N = n;
  pb.K = k;
  pb.Mp = (m + OZ_BM - 1) / OZ_BM * OZ_BM;
  pb.Np = (n + OZ_BN - 1) / OZ_BN * OZ_BN;
  pb.Kp = k <= 0 ? OZ_BK : (k + OZ_BK - 1) / OZ_BK * OZ_BK;
  pb.crt = 1;
  pb.w = w;
  pb.L = L;
  pb.mplanes = L;
  pb.s = slices;
  pb.sr = 2;
  OzPairList& pl = plan.crt;
  for (int l = 0; l < L; ++l) {
    pl.pa[l] = pl.pb[l] = (int8_t)l;
    pl.gstart[l] = (int16_t)l;
    pl.gt[l] = (int8_t)l;
  }
  pl.gstart[L] = (int16_t)L;
  pl.npairs = pl.ngroups = L;
  // scratch: planes A, planes B, residues, rowmax, E, F, flag
  const size_t bA = al256d((size_t)L * pb.Mp * pb.Kp * 2), bB = al256d((size_t)L * pb.Np * pb.Kp * 2),
               bR = al256d((size_t)L * pb.Np * pb.Mp), bM = al256d(8 * (size_t)pb.Mp),
               bE = al256d(4 * (size_t)pb.Mp), bF = al256d(4 * (size_t)pb.Np), bG = 256;
  const size_t total = bA + bB + bR + bM + bE + bF + bG;
  Scratch buf;
  uint8_t* base;
  if (static_scratch) {
    if (total > static_bytes) {
      set_error("ddgemm: needs %zu bytes of scratch, more than the %zu available", total,
                static_bytes);
      return VCPCU_ERR_INVALID_ARG;
    }
    base = (uint8_t*)static_scratch;
  } else {
    int st = buf.alloc(total, s);
    if (st) return st;
    base = (uint8_t*)buf.ptr;
  }
  OzWorkspace ws;
  memset(&ws, 0, sizeof(ws));
  ws.a_mid = (uint16_t*)base;
  ws.b_mid = (uint16_t*)(base + bA);
  ws.res = base + bA + bB;
  unsigned long long* rowmax = (unsigned long long*)(base + bA + bB + bR);
  int* E = (int*)(base + bA + bB + bR + bM);
  int* F = (int*)(base + bA + bB + bR + bM + bE);
  ws.flag = (int*)(base + bA + bB + bR + bM + bE + bF);
  ws.E3 = E;
  ws.F2 = F;
  int st;
  {
    PhaseTimer t(0, s);
    st = dd_prepare(m, n, k, pb.Mp, pb.Np, pb.Kp, L, w, A, lda, B, ldb, rowmax, E, F, ws.a_mid,
                    ws.b_mid, ws.flag, s);
    if (st) return st;
  }
  {
    PhaseTimer t(3, s);
    if ((st = oz_run_gemm(plan, OZ_CRT, ws, nullptr, 0, s))) return st;
  }
  oz_profile_add_flops(2LL * m * n * (long long)(k > 0 ? k : 0) * L);
  {
    PhaseTimer t(4, s);
    dim3 grid((m + 255) / 256, n < 65535 ? n : 65535);
    dd_crt_assemble_kernel<<<grid, 256, 0, s>>>(m, n, k, pb.Mp, L, w, ws.res,
                                                (size_t)pb.Np * pb.Mp, E, F, C, ldc, Cerr, lde,
                                                ws.flag, cc);
    VCPCU_LAUNCH_CHECK("dd_crt_assemble_kernel");
  }
  oz_merge_status(ws.flag, s);
  return VCPCU_OK;
}

}  // namespace vcpcu
