// swfp.cuh -- binary64 midrad on the integer pipe.
//
// GB300 issues FP64 at 1/64 of the FP32 rate, so the operand preparation of
// the tensor-core form (one kv midrad per interval entry) is bound by the
// FP64 pipe when it uses FP64 instructions.  (A single FP64 instruction per
// entry beside integer-bound work is cheaper on the FP64 pipe, which runs in
// parallel: the upward additions |m| + r of the splits and of the radius
// term stay FP64 instructions.)  The functions below compute the
// same bits with integer operations for the common case -- both endpoints
// normal, of one sign, binary exponents at most one apart (an interval
// narrower than its midpoint) -- and fall back to the FP64 instructions
// otherwise.  Every result equals the hardware result bit for bit:
//   m = RN(lo + up) * 0.5  (kv midpoint; RN(lo/2 + up/2) if lo + up overflows)
//   r = max(RU(m - lo), RU(up - m))
//   p = RU(|m| + r)
#pragma once
#include <cstdint>

namespace vcpcu {

// Bit pattern <-> double through an opaque move: the compiler then cannot
// fold the integer code below back into FP64 instructions (a sign-bit mask
// into an FP64 absolute value, a zero test into an FP64 comparison).
__device__ __forceinline__ unsigned long long sw_bits(double x) {
  unsigned long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}
__device__ __forceinline__ double sw_double(unsigned long long b) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(b));
  return x;
}
// -x by flipping the sign bit
__device__ __forceinline__ double sw_neg(double x) { return sw_double(sw_bits(x) ^ (1ULL << 63)); }
// finite (neither Inf nor NaN), from the exponent field
__device__ __forceinline__ bool sw_finite(double x) {
  return ((sw_bits(x) >> 52) & 0x7ff) != 0x7ff;
}

// Comparisons with zero and the kv absolute value on bit patterns (GB300
// runs FP64 compares and negations on its narrow FP64 pipe).  NaN compares
// false, as in IEEE.
__device__ __forceinline__ bool sw_isnan_b(unsigned long long b) {
  return (b & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL;
}
__device__ __forceinline__ bool sw_ge0_b(unsigned long long b) {  // x >= 0
  return !sw_isnan_b(b) && ((b >> 63) == 0 || b == 0x8000000000000000ULL);
}
__device__ __forceinline__ bool sw_le0_b(unsigned long long b) {  // x <= 0
  return !sw_isnan_b(b) && ((b >> 63) != 0 || b == 0);
}
// kv abs([lo, up]): [lo, up] if lo >= 0; [-up, -lo] if up <= 0; else
// [+0, std::max(-lo, up)] (std::max(a, b) = a < b ? b : a).
// Branch-free (selects only), so that lanes of a warp taking different cases
// do not diverge.
__device__ __forceinline__ void sw_abs_iv(double lo, double up, double& alo, double& aup) {
  const unsigned long long bl = sw_bits(lo), bu = sw_bits(up), S = 1ULL << 63;
  const bool ge = sw_ge0_b(bl), le = sw_le0_b(bu);
  const unsigned long long a = bl ^ S;  // -lo
  // lo < 0 < up (or a NaN): -lo < up compares two positive doubles
  const unsigned long long mx = (!sw_isnan_b(a) && !sw_isnan_b(bu) && a < bu) ? bu : a;
  alo = sw_double(ge ? bl : (le ? (bu ^ S) : 0ULL));
  aup = sw_double(ge ? bu : (le ? a : mx));
}
__device__ __forceinline__ double sw_abs_sup(double lo, double up) {
  double alo, aup;
  sw_abs_iv(lo, up, alo, aup);
  return aup;
}

// RU(X * 2^(g - 1075)) for an integer X > 0 (< 2^63) as a normal double:
// returns false if the result would be subnormal.  Also returns the rounded
// value as an integer multiple of 2^(g - 1075) in *Xr (exact when X has at
// most 53 significant bits).
__device__ __forceinline__ bool sw_ru_int(unsigned long long X, int g, double* out,
                                          unsigned long long* Xr) {
  const int bd = 64 - __clzll(X);
  unsigned long long M;
  int B;
  if (bd <= 53) {
    M = X << (53 - bd);
    B = g - (53 - bd);
    *Xr = X;
  } else {
    const int s = bd - 53;
    M = X >> s;
    B = g + s;
    if (X & ((1ULL << s) - 1)) {
      ++M;
      if (M >> 53) {
        M >>= 1;
        ++B;
      }
    }
    *Xr = M << (B - g);
  }
  if (B < 1 || B > 2046) return false;
  *out = sw_double(((unsigned long long)B << 52) | (M & ((1ULL << 52) - 1)));
  return true;
}

// Integer-pipe midrad of [lo, up] (see the file comment); false: not the
// common case, nothing written.
__device__ __forceinline__ bool sw_midrad_fast(double lo, double up, double& m, double& r,
                                               double& p) {
  const unsigned long long bl = sw_bits(lo), bu = sw_bits(up);
  const int sl = (int)(bl >> 63), su = (int)(bu >> 63);
  const int el = (int)((bl >> 52) & 0x7ff), eu = (int)((bu >> 52) & 0x7ff);
  if (sl != su || el == 0 || eu == 0 || el > 2045 || eu > 2045) return false;
  const int e = el > eu ? el : eu;
  if (e - (el < eu ? el : eu) > 1) return false;
  const unsigned long long H = 1ULL << 52;
  // magnitudes in units 2^(e - 1076): exact (shift by 0 or 1)
  const unsigned long long Xl = ((bl & (H - 1)) | H) << (el - e + 1);
  const unsigned long long Xu = ((bu & (H - 1)) | H) << (eu - e + 1);
  // |lo + up| in units 2^(e - 1076) = |midpoint| in units u = 2^(e - 1077)
  const unsigned long long S = Xl + Xu;  // 2^53 + 2^52 <= S < 2^55
  const int sh = (64 - __clzll(S)) - 53;  // 1 or 2
  unsigned long long M = S >> sh;
  const unsigned long long rem = S & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
  if (rem > half || (rem == half && (M & 1ULL))) ++M;
  int B = sh + e - 2;  // value M 2^(B - 1075)
  int shm = sh;
  if (M >> 53) {
    M >>= 1;
    ++B;
    ++shm;
  }
  if (B < 1 || B > 2046) return false;
  const unsigned long long Xm = M << shm;  // |m| in units u
  const unsigned long long L2 = Xl << 1, U2 = Xu << 1;
  // m - lo and up - m as magnitudes in units u (both >= 0: m lies in [lo, up])
  const unsigned long long D1 = sl ? L2 - Xm : Xm - L2;
  const unsigned long long D2 = sl ? Xm - U2 : U2 - Xm;
  const unsigned long long D = D1 > D2 ? D1 : D2;
  double rv = 0.0;
  unsigned long long Rr = 0;
  if (D && !sw_ru_int(D, e - 2, &rv, &Rr)) return false;
  double pv;
  unsigned long long Pr;
  if (!sw_ru_int(Xm + Rr, e - 2, &pv, &Pr)) return false;
  m = sw_double(((unsigned long long)sl << 63) | ((unsigned long long)B << 52) | (M & (H - 1)));
  r = rv;
  p = pv;
  return true;
}

// The same three values with the FP64 instructions (every finite input).
__device__ __forceinline__ void sw_midrad_hw(double lo, double up, double& m, double& r,
                                             double& p) {
  const double s = __dadd_rn(lo, up);
  if (sw_finite(s))
    m = __dmul_rn(s, 0.5);
  else
    m = __dadd_rn(__dmul_rn(lo, 0.5), __dmul_rn(up, 0.5));
  r = fmax(__dsub_ru(m, lo), __dsub_ru(up, m));
  p = __dadd_ru(fabs(m), r);
}

// The FP64 fallbacks are out of line: inlined, the compiler may issue their
// first FP64 instruction speculatively on the common path.
static __device__ __noinline__ void sw_midrad_slow(double lo, double up, double& m, double& r,
                                            double& p) {
  sw_midrad_hw(lo, up, m, r, p);
}

__device__ __forceinline__ void sw_midrad(double lo, double up, double& m, double& r,
                                          double& p) {
  if (!sw_midrad_fast(lo, up, m, r, p)) sw_midrad_slow(lo, up, m, r, p);
}

}  // namespace vcpcu
