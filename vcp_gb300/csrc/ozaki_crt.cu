// ozaki_crt.cu -- reassembly of the CRT (Ozaki-II) form of the midpoint
// product and the final enclosure.
//
// For each entry the slice GEMM left the residues c_l = (A'B')(i,j) mod m_l
// (l < L) of the exact integer product of the w-bit operands
// A' = round(mA 2^(w-E_i)), B' = round(mB 2^(w-F_j)).  Chinese remaindering
// gives X = sum_l c_l Q_l mod M (Q_l = (M/m_l) ((M/m_l)^-1 mod m_l)), taken
// in (-M/2, M/2]; since prod m_l > 2 |A'B'|, X = (A'B')(i,j) exactly.  Then
//   mA mB = 2^(E+F-2w) X + ΔA mB + Â ΔB,   |ΔA| <= 2^(E-w-1), |ΔB| <= 2^(F-w-1),
//   |ΔA mB| <= 2^(E-w-1) beta_j,   |Â ΔB| <= 2^(E+F-2w-1) sum_k |A'(i,k)|,
// and the enclosure is [RD(2^(E+F-2w) X) - e, RU(2^(E+F-2w) X) + e] with
// e = RU(RU(trunc) + T(i,j)), T the upper bound of the radius term.
#include "common.cuh"
#include "ozaki.cuh"
#include "ozaki_common.cuh"

namespace vcpcu {

namespace {

struct CrtConst {
  uint32_t Q[16][4];
  uint32_t M[4];
  double Md;
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

// r (5 limbs of 32 bits, little endian) >= m (4 limbs)?
__device__ __forceinline__ bool ge_M(const uint32_t* r, const uint32_t* m) {
  if (r[4]) return true;
  for (int t = 3; t >= 0; --t) {
    if (r[t] != m[t]) return r[t] > m[t];
  }
  return true;
}

__device__ __forceinline__ void sub_M(uint32_t* r, const uint32_t* m) {
  unsigned long long borrow = 0;
  for (int t = 0; t < 5; ++t) {
    const unsigned long long mt = t < 4 ? m[t] : 0u;
    const unsigned long long d = (unsigned long long)r[t] - mt - borrow;
    r[t] = (uint32_t)d;
    borrow = (d >> 63) & 1ULL;
  }
}

__device__ __forceinline__ void add_M(uint32_t* r, const uint32_t* m) {
  unsigned long long carry = 0;
  for (int t = 0; t < 5; ++t) {
    const unsigned long long mt = t < 4 ? m[t] : 0u;
    const unsigned long long s = (unsigned long long)r[t] + mt + carry;
    r[t] = (uint32_t)s;
    carry = s >> 32;
  }
}

// Directed conversion of (-1)^neg * mag * 2^e (mag: 4 limbs) to double.
__device__ __forceinline__ void big_to_dir(const uint32_t* mag, int neg, int e, double& lo,
                                           double& up) {
  int top = 3;
  while (top >= 0 && mag[top] == 0) --top;
  if (top < 0) {
    lo = up = 0.0;
    return;
  }
  const int bl = 32 * top + (32 - __clz(mag[top]));  // bit length, 1..128
  unsigned long long t;
  int sh = 0;
  bool sticky = false;
  if (bl <= 64) {
    t = (unsigned long long)mag[0] | ((unsigned long long)mag[1] << 32);
  } else {
    sh = bl - 64;
    // t = mag >> sh (top 64 bits), sticky = any bit below sh
    const int wq = sh >> 5, bq = sh & 31;
    unsigned long long w0 = mag[wq], w1 = (wq + 1 < 4) ? mag[wq + 1] : 0u,
                       w2 = (wq + 2 < 4) ? mag[wq + 2] : 0u;
    unsigned long long lo64 = w0 | (w1 << 32);
    t = bq ? ((lo64 >> bq) | (w2 << (64 - bq))) : lo64;
    for (int q = 0; q < wq; ++q) sticky |= mag[q] != 0;
    if (bq) sticky |= (mag[wq] & ((1u << bq) - 1u)) != 0;
  }
  if (sticky) t |= 1ULL;
  const double a_dn = __ull2double_rd(t), a_up = __ull2double_ru(t);
  const int ex = e + sh;
  if (!neg) {
    lo = scale_dir2(a_dn, ex, false);
    up = scale_dir2(a_up, ex, true);
  } else {
    lo = -scale_dir2(a_up, ex, true);
    up = -scale_dir2(a_dn, ex, false);
  }
}

__global__ void __launch_bounds__(256)
oz_crt_assemble_kernel(int M, int N, int Mp, int L, int w, const uint8_t* __restrict__ res,
                       size_t plane, const int* __restrict__ E3, const int* __restrict__ F2,
                       const unsigned long long* __restrict__ asum,
                       const double* __restrict__ beta, const double* __restrict__ T,
                       double* __restrict__ C, long ldc, const int* __restrict__ flag,
                       const __grid_constant__ CrtConst cc) {
  const bool nonfinite = flag[0] != 0 || flag[1] != 0;
  const long total = (long)M * N;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % M), j = (int)(idx / M);
    const size_t e = (size_t)j * Mp + i;
    const int Ei = E3[3 * i], Fj = F2[2 * j];
    double lo = 0.0, up = 0.0, tr = 0.0;
    if (Ei != OZ_ZERO_EXP && Fj != OZ_ZERO_EXP) {
      unsigned long long s[4] = {0, 0, 0, 0};
      for (int l = 0; l < L; ++l) {
        const unsigned long long c = res[(size_t)l * plane + e];
#pragma unroll
        for (int t = 0; t < 4; ++t) s[t] += c * cc.Q[l][t];
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
      // q = floor(S / M) estimated from the top limbs, then corrected
      const double Sd = (double)r[4] * 0x1p128 + (double)r[3] * 0x1p96 + (double)r[2] * 0x1p64 +
                        (double)r[1] * 0x1p32 + (double)r[0];
      unsigned int q = (unsigned int)(Sd / cc.Md);
      if (q) {
        // r -= q * M
        unsigned long long qm[5];
        unsigned long long c2 = 0;
        for (int t = 0; t < 4; ++t) {
          const unsigned long long v = (unsigned long long)q * cc.M[t] + c2;
          qm[t] = (uint32_t)v;
          c2 = v >> 32;
        }
        qm[4] = c2;
        unsigned long long borrow = 0;
        for (int t = 0; t < 5; ++t) {
          const unsigned long long d = (unsigned long long)r[t] - qm[t] - borrow;
          r[t] = (uint32_t)d;
          borrow = (d >> 63) & 1ULL;
        }
        for (int it = 0; it < 4 && borrow; ++it) {  // q was too large
          add_M(r, cc.M);
          borrow = (r[4] >> 31) & 1u;  // still negative (two's complement in 5 limbs)
        }
      }
      for (int it = 0; it < 4 && ge_M(r, cc.M); ++it) sub_M(r, cc.M);
      // centre: X = r if 2r < M, else r - M (magnitude M - r)
      uint32_t twice[5];
      unsigned long long cy = 0;
      for (int t = 0; t < 5; ++t) {
        const unsigned long long v = ((unsigned long long)r[t] << 1) + cy;
        twice[t] = (uint32_t)v;
        cy = v >> 32;
      }
      int neg = 0;
      uint32_t mag[4];
      if (ge_M(twice, cc.M)) {
        neg = 1;
        unsigned long long b = 0;
        for (int t = 0; t < 4; ++t) {
          const unsigned long long d = (unsigned long long)cc.M[t] - r[t] - b;
          mag[t] = (uint32_t)d;
          b = (d >> 63) & 1ULL;
        }
      } else {
        for (int t = 0; t < 4; ++t) mag[t] = r[t];
      }
      big_to_dir(mag, neg, Ei + Fj - 2 * w, lo, up);
      // truncation bound
      const double sA = __fma_ru((double)asum[2 * i + 0], 0x1p32, (double)asum[2 * i + 1]);
      const double t1 = scale_dir2(beta[j], Ei - w - 1, true);
      const double t2 = scale_dir2(sA, Ei + Fj - 2 * w - 1, true);
      tr = __dadd_ru(t1, t2);
    }
    const double err = __dadd_ru(tr, T[e]);
    double clo = __dsub_rd(lo, err), cup = __dadd_ru(up, err);
    if (nonfinite) clo = cup = __longlong_as_double(0x7ff8000000000000LL);
    C[2 * ((size_t)i + (size_t)j * ldc)] = clo;
    C[2 * ((size_t)i + (size_t)j * ldc) + 1] = cup;
  }
}

}  // namespace

int oz_crt_assemble(const OzPlan& plan, const OzWorkspace& ws, double* C, long ldc,
                    cudaStream_t st) {
  const OzProblem& pb = plan.pb;
  CrtConst cc;
  memset(&cc, 0, sizeof(cc));
  for (int l = 0; l < pb.L; ++l)
    for (int t = 0; t < 4; ++t) cc.Q[l][t] = plan.Q[l][t];
  for (int t = 0; t < 4; ++t) cc.M[t] = plan.Mlimb[t];
  cc.Md = (double)cc.M[3] * 0x1p96 + (double)cc.M[2] * 0x1p64 + (double)cc.M[1] * 0x1p32 +
          (double)cc.M[0];
  const long total = (long)pb.M * pb.N;
  long blocks = (total + 255) / 256;
  if (blocks > 152L * 64) blocks = 152L * 64;
  if (blocks < 1) blocks = 1;
  oz_crt_assemble_kernel<<<(int)blocks, 256, 0, st>>>(
      pb.M, pb.N, pb.Mp, pb.L, pb.w, ws.res, (size_t)pb.Np * pb.Mp, ws.E3, ws.F2, ws.asum,
      ws.beta, ws.T, C, ldc, ws.flag, cc);
  VCPCU_LAUNCH_CHECK("oz_crt_assemble_kernel");
  return VCPCU_OK;
}

}  // namespace vcpcu
