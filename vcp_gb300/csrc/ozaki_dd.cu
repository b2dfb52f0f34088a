// ozaki_dd.cu -- double-double GEMM (the vcp::pddcuda policy, pddblas
// semantics: vcp/pddblas.hpp:318-409) on the tensor cores.
//
// pddblas splits each dd operand into double slices, multiplies every slice
// pair with dgemm and accumulates the exact products in dd
// (pddblas_assist::split_row / split_col / ozaki_acc, vcp/pddblas.hpp:82-193).
// Here each dd entry hi + lo is scaled per row (A) / column (B) to a w-bit
// integer (w = 8 * slices, default 104 bits), the integer product A'B' is
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
  double Md;
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
  c->Md = 0.0;
  for (int t = DDL - 1; t >= 0; --t) c->Md = c->Md * 4294967296.0 + (double)c->M[t];
  return 0;
}

// ---- device ---------------------------------------------------------------
__device__ __forceinline__ double pow2(int e) {  // exact for -1022 <= e <= 1023
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// mag (DDL limbs) -> (top 64 bits with sticky, shift)
__device__ __forceinline__ unsigned long long top64(const uint32_t* mag, int bl, int& sh) {
  if (bl <= 64) {
    sh = 0;
    return (unsigned long long)mag[0] | ((unsigned long long)mag[1] << 32);
  }
  sh = bl - 64;
  const int wq = sh >> 5, bq = sh & 31;
  const unsigned long long w0 = mag[wq], w1 = (wq + 1 < DDL) ? mag[wq + 1] : 0u,
                           w2 = (wq + 2 < DDL) ? mag[wq + 2] : 0u;
  const unsigned long long lo64 = w0 | (w1 << 32);
  unsigned long long t = bq ? ((lo64 >> bq) | (w2 << (64 - bq))) : lo64;
  bool sticky = false;
  for (int q = 0; q < wq; ++q) sticky |= mag[q] != 0;
  if (bq) sticky |= (mag[wq] & ((1u << bq) - 1u)) != 0;
  if (sticky) t |= 1ULL;
  return t;
}

__device__ __forceinline__ int bitlen(const uint32_t* mag) {
  for (int t = DDL - 1; t >= 0; --t)
    if (mag[t]) return 32 * t + (32 - __clz(mag[t]));
  return 0;
}

__global__ void __launch_bounds__(256)
dd_crt_assemble_kernel(int M, int N, int K, int Mp, int L, int w, const uint8_t* __restrict__ res,
                       size_t plane, const int* __restrict__ E, const int* __restrict__ F,
                       double* __restrict__ C, long ldc, double* __restrict__ Cerr, long lde,
                       const int* __restrict__ flag, const __grid_constant__ DdCrt cc) {
  const bool bad = flag[0] != 0 || flag[1] != 0;
  const long total = (long)M * N;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % M), j = (int)(idx / M);
    const int Ei = E[i], Fj = F[j];
    double hi = 0.0, lo = 0.0, err = 0.0;
    if (Ei != OZ_ZERO_EXP && Fj != OZ_ZERO_EXP) {
      const size_t e = (size_t)j * Mp + i;
      unsigned long long s[DDL];
#pragma unroll
      for (int t = 0; t < DDL; ++t) s[t] = 0;
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
      double Sd = 0.0;
      for (int t = DDL; t >= 0; --t) Sd = Sd * 4294967296.0 + (double)r[t];
      const unsigned int q = (unsigned int)(Sd / cc.Md);
      // r -= q M, then correct to [0, M)
      {
        unsigned long long c2 = 0, borrow = 0;
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
          for (int t = 0; t <= DDL; ++t) {
            const unsigned long long v = (unsigned long long)r[t] + (t < DDL ? cc.M[t] : 0u) + cy;
            r[t] = (uint32_t)v;
            cy = v >> 32;
          }
        }
        for (int it = 0; it < 4; ++it) {  // r >= M: subtract
          bool ge = r[DDL] != 0;
          if (!ge) {
            ge = true;
            for (int t = DDL - 1; t >= 0; --t)
              if (r[t] != cc.M[t]) {
                ge = r[t] > cc.M[t];
                break;
              }
          }
          if (!ge) break;
          unsigned long long b = 0;
          for (int t = 0; t <= DDL; ++t) {
            const unsigned long long d =
                (unsigned long long)r[t] - (t < DDL ? cc.M[t] : 0u) - b;
            r[t] = (uint32_t)d;
            b = (d >> 63) & 1ULL;
          }
        }
      }
      // centre: X = r (2r < M) or r - M
      int neg = 0;
      uint32_t mag[DDL];
      {
        bool ge = false;  // 2r >= M ?
        uint32_t tw[DDL + 1];
        unsigned long long cy = 0;
        for (int t = 0; t < DDL; ++t) {
          const unsigned long long v = ((unsigned long long)r[t] << 1) + cy;
          tw[t] = (uint32_t)v;
          cy = v >> 32;
        }
        tw[DDL] = (uint32_t)cy;
        ge = tw[DDL] != 0;
        if (!ge) {
          ge = true;
          for (int t = DDL - 1; t >= 0; --t)
            if (tw[t] != cc.M[t]) {
              ge = tw[t] > cc.M[t];
              break;
            }
        }
        if (ge) {
          neg = 1;
          unsigned long long b = 0;
          for (int t = 0; t < DDL; ++t) {
            const unsigned long long d = (unsigned long long)cc.M[t] - r[t] - b;
            mag[t] = (uint32_t)d;
            b = (d >> 63) & 1ULL;
          }
        } else {
          for (int t = 0; t < DDL; ++t) mag[t] = r[t];
        }
      }
      // dd of mag * 2^ex: hi = RN, lo = RN of the exact remainder
      const int ex = Ei + Fj - 2 * w;
      const int bl = bitlen(mag);
      bool range_ok = true;
      if (bl > 0) {
        int sh;
        const unsigned long long t = top64(mag, bl, sh);
        const double hm = __ull2double_rn(t);  // <= 2^64, 53 significant bits
        if (ex + sh < -1022 || ex + sh + 64 > 1023) range_ok = false;
        // remainder Y = mag - round(hm) << sh, as a signed 2-word value
        // (|Y| < 2^(sh + 11)); exact in 128 bits while sh <= 100
        unsigned __int128 H = (unsigned __int128)hm;
        // mag >> 0 restricted to the low (sh + 12) bits region: compute Y via
        // full-width subtraction of H << sh from mag
        uint32_t hsh[DDL];
        for (int q = 0; q < DDL; ++q) hsh[q] = 0;
        {
          const int wq = sh >> 5, bq = sh & 31;
          unsigned __int128 Hs = H;
          // place H (<= 65 bits) shifted by bq into limbs starting at wq
          unsigned __int128 v = Hs << bq;  // <= 97 bits
          for (int q = 0; q < 4 && wq + q < DDL; ++q) hsh[wq + q] = (uint32_t)(v >> (32 * q));
        }
        // Y = mag - hsh (signed)
        uint32_t y[DDL];
        unsigned long long b = 0;
        for (int q = 0; q < DDL; ++q) {
          const unsigned long long d = (unsigned long long)mag[q] - hsh[q] - b;
          y[q] = (uint32_t)d;
          b = (d >> 63) & 1ULL;
        }
        int yneg = (int)b;
        if (yneg) {  // negate two's complement
          unsigned long long cy = 1;
          for (int q = 0; q < DDL; ++q) {
            const unsigned long long v = (unsigned long long)(~y[q]) + cy;
            y[q] = (uint32_t)v;
            cy = v >> 32;
          }
        }
        double hval = range_ok ? hm * pow2(ex + sh) : 0.0;
        double lval = 0.0;
        const int ybl = bitlen(y);
        if (ybl > 0) {
          int ysh;
          const unsigned long long yt = top64(y, ybl, ysh);
          const double ym = __ull2double_rn(yt);
          const int ye = ex + ysh;
          if (ye < -1022 || ye + 64 > 1023)
            range_ok = false;
          else
            lval = ym * pow2(ye);
          if (yneg) lval = -lval;
        }
        hi = neg ? -hval : hval;
        lo = neg ? -lval : lval;
        // conversion error <= ulp(lo) (<= |lo| 2^-52) + 2^-1074
        err = __fma_ru(fabs(lo), 0x1p-52, 0x1p-1074);
      }
      // truncation of the operands to w-bit integers: K 2^(E+F-w) (1 + 2^-40)
      const double kf = __dmul_ru((double)(K > 0 ? K : 0), 1.0 + 0x1p-40);
      int et = Ei + Fj - w;
      double tr = kf;
      while (et > 1023) { tr = __dmul_ru(tr, 0x1p1023); et -= 1023; }
      while (et < -1022) { tr = __dmul_ru(tr, 0x1p-1022); et += 1022; }
      tr = __dmul_ru(tr, pow2(et));
      err = __dadd_ru(err, tr);
      if (!range_ok) err = INFINITY;
    }
    if (bad) hi = lo = err = __longlong_as_double(0x7ff8000000000000LL);
    C[2 * ((size_t)i + (size_t)j * ldc)] = hi;
    C[2 * ((size_t)i + (size_t)j * ldc) + 1] = lo;
    if (Cerr) Cerr[(size_t)i + (size_t)j * lde] = err;
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
  int w = 8 * (slices > 0 ? slices : 13), L = 0;
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
  long blocks = ((long)m * n + 255) / 256;
  if (blocks > 152L * 64) blocks = 152L * 64;
  if (blocks < 1) blocks = 1;
  {
    PhaseTimer t(4, s);
    dd_crt_assemble_kernel<<<(int)blocks, 256, 0, s>>>(m, n, k, pb.Mp, L, w, ws.res,
                                                       (size_t)pb.Np * pb.Mp, E, F, C, ldc, Cerr,
                                                       lde, ws.flag, cc);
    VCPCU_LAUNCH_CHECK("dd_crt_assemble_kernel");
  }
  oz_merge_status(ws.flag, s);
  return VCPCU_OK;
}

}  // namespace vcpcu
