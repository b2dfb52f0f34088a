// ozaki_common.cuh -- integer slicing shared by the split kernels and the
// slice-GEMM epilogue (host- and device-callable, bit-for-bit the same as the
// host model in oracle/ozaki_model.c).
//
// Slicing (the Ozaki scheme, error-free splitting; cf. the reference's
// pddblas_assist::split_row / split_col, vcp/pddblas.hpp:82-154, which
// slices with sigma = 2^(e+s) per row/column): every row i of a left factor
// (column j of a right factor) gets an exponent E with max |x| <= 2^(E-1).
// x * 2^(8s-E) is rounded to an integer N (to nearest-even for two-sided
// products, upward for the non-negative radius factors) and N is written
// as s balanced base-256 digits d_1..d_s, each in [-128, 128], so that
//     x = 2^E * (sum_p d_p 2^(-8p)) + remainder.
// Every digit is an integer of at most 8 significant bits, hence exact in
// bf16, every digit product is at most 2^14, and a sum of up to 1024 such
// products is an integer of magnitude <= 2^24, exact in the fp32 tensor-core
// accumulator.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define OZ_HD __host__ __device__ __forceinline__
#else
#define OZ_HD inline
#endif

namespace vcpcu {

constexpr int OZ_ZERO_EXP = -30000;   // exponent sentinel of an all-zero row/column
constexpr int OZ_CHUNK = 1024;        // k elements per exact fp32 accumulation chunk
constexpr int OZ_FOLD_CHUNKS = 64;    // chunks per int32 fold (64 * 2^24 = 2^30)

OZ_HD uint64_t oz_bits(double x) {
#ifdef __CUDA_ARCH__
  uint64_t b;  // an opaque move: keeps integer tests of the bits on the integer pipe
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}

// x == +-0 tested on the bit pattern (an FP64 comparison would issue on the
// narrow FP64 pipe of GB300).
OZ_HD bool oz_zero(double x) { return (oz_bits(x) << 1) == 0; }
// |x| by clearing the sign bit (integer pipe).
OZ_HD double oz_abs(double x) {
  const uint64_t b = oz_bits(x) & 0x7fffffffffffffffULL;
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double r;
  memcpy(&r, &b, 8);
  return r;
#endif
}

// E such that |x| <= 2^(E-1) for the largest magnitude `amax` (>= 0, finite);
// OZ_ZERO_EXP for amax == 0.
OZ_HD int oz_exponent(double amax) {
  uint64_t b = oz_bits(amax);
  int be = (int)((b >> 52) & 0x7ff);
  uint64_t mant = b & ((1ULL << 52) - 1);
  if (be == 0 && mant == 0) return OZ_ZERO_EXP;
  if (be == 0) {  // subnormal: amax < 2^(bitlen(mant) - 1074)
    int bl = 0;
    while (mant) {
      mant >>= 1;
      ++bl;
    }
    return bl - 1074 + 1;
  }
  return be - 1021;  // amax < 2^(be-1022)
}

// N = x * 2^(bits - E) rounded to an integer: to nearest-even (up == 0) or
// toward +inf (up == 1; used for x >= 0).  Requires |x| <= 2^(E-1), so
// |N| <= 2^(bits-1) (bits <= 96 keeps N within an int128).
OZ_HD __int128 oz_scaled_int_bits(double x, int E, int bits, int up) {
  uint64_t b = oz_bits(x);
  const int neg = (int)(b >> 63);
  const int be = (int)((b >> 52) & 0x7ff);
  uint64_t mant = b & ((1ULL << 52) - 1);
  if (be == 0 && mant == 0) return 0;
  int ex;
  if (be == 0) {
    ex = -1074;
  } else {
    mant |= 1ULL << 52;
    ex = be - 1075;
  }
  const int sh = ex + bits - E;
  unsigned __int128 N;
  if (sh >= 0) {
    N = (unsigned __int128)mant << sh;
  } else {
    const int r = -sh;
    uint64_t q;
    bool rem_nz, above_half, at_half;
    if (r >= 64) {
      q = 0;
      rem_nz = mant != 0;
      above_half = false;
      at_half = false;
    } else {
      q = mant >> r;
      const uint64_t rem = mant & ((1ULL << r) - 1);
      const uint64_t half = 1ULL << (r - 1);
      rem_nz = rem != 0;
      above_half = rem > half;
      at_half = rem == half;
    }
    if (up) {
      // ceil of the magnitude for x >= 0; for x < 0 (not used) truncate
      if (!neg && rem_nz) q += 1;
    } else {
      if (above_half || (at_half && (q & 1))) q += 1;
    }
    N = q;
  }
  return neg ? -(__int128)N : (__int128)N;
}

// The same for bits <= 62 in 64-bit arithmetic (|N| <= 2^(bits-1)).
OZ_HD long long oz_scaled_int64(double x, int E, int bits, int up) {
  uint64_t b = oz_bits(x);
  const int neg = (int)(b >> 63);
  const int be = (int)((b >> 52) & 0x7ff);
  uint64_t mant = b & ((1ULL << 52) - 1);
  if (be == 0 && mant == 0) return 0;
  int ex;
  if (be == 0) {
    ex = -1074;
  } else {
    mant |= 1ULL << 52;
    ex = be - 1075;
  }
  const int sh = ex + bits - E;
  uint64_t N;
  if (sh >= 0) {
    N = mant << sh;
  } else {
    const int r = -sh;
    uint64_t q;
    bool rem_nz, above_half, at_half;
    if (r >= 64) {
      q = 0;
      rem_nz = mant != 0;
      above_half = false;
      at_half = false;
    } else {
      q = mant >> r;
      const uint64_t rem = mant & ((1ULL << r) - 1);
      const uint64_t half = 1ULL << (r - 1);
      rem_nz = rem != 0;
      above_half = rem > half;
      at_half = rem == half;
    }
    if (up) {
      if (!neg && rem_nz) q += 1;
    } else {
      if (above_half || (at_half && (q & 1))) q += 1;
    }
    N = q;
  }
  return neg ? -(long long)N : (long long)N;
}

// Digit form: x * 2^(8s - E) (s base-256 digits).
OZ_HD __int128 oz_scaled_int(double x, int E, int s, int up) {
  return oz_scaled_int_bits(x, E, 8 * s, up);
}

// Moduli of the CRT (Ozaki-II) form: pairwise coprime, at most 256, so a
// residue taken in the symmetric range fits in [-128, 127] (exact in bf16).
constexpr int OZ_MAX_MODULI = 32;
constexpr int OZ_MODULI[OZ_MAX_MODULI] = {256, 255, 253, 251, 247, 241, 239, 233,
                                          229, 227, 223, 217, 211, 199, 197, 193,
                                          191, 181, 179, 173, 167, 163, 157, 151,
                                          149, 139, 137, 131, 127, 113, 109, 107};
// The interval (double) CRT form uses the first 16 (product < 2^128).
constexpr int OZ_MAX_MODULI_128 = 16;

// Symmetric residue of (neg ? -a : a) modulo m (2 <= m <= 256), in
// [-floor(m/2), ceil(m/2) - 1].
OZ_HD int oz_sym_residue(unsigned long long a, int neg, int m) {
  unsigned long long r = a % (unsigned long long)m;
  if (neg && r) r = (unsigned long long)m - r;
  int rs = (int)r;
  if (2 * rs >= m) rs -= m;
  return rs;
}

// Balanced base-256 digits of N, most significant first: d[0] = d_1.
OZ_HD void oz_digits(__int128 N, int s, int* d) {
  for (int p = s - 1; p >= 1; --p) {
    const int lo = (int)((uint64_t)(N + 128) & 255ULL) - 128;
    d[p] = lo;
    N = (N - lo) >> 8;
  }
  d[0] = (int)N;
}

// bf16 bit pattern of an integer |v| <= 256 (exact).
OZ_HD uint16_t oz_bf16_of_int(int v) {
  if (v == 0) return 0;
  uint16_t sign = v < 0 ? 0x8000 : 0;
  unsigned a = (unsigned)(v < 0 ? -v : v);
  int e = 0;  // a = 1.f * 2^e, e <= 8
  while ((a >> (e + 1)) != 0) ++e;
  unsigned frac = (e <= 7 ? (a << (7 - e)) : (a >> (e - 7))) & 0x7f;  // 7 explicit bits
  return (uint16_t)(sign | ((unsigned)(e + 127) << 7) | frac);
}

// Paired FP32 arithmetic (sm_100 and later): two floats in one 64-bit
// register pair, the first in the low half; each instruction rounds each
// half to nearest exactly as the scalar instruction does, so a pair gives
// the bits of two scalar evaluations in half the issue slots.
__device__ __forceinline__ unsigned long long f32x2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ unsigned long long fma_x2(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ unsigned long long mul_x2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long add_x2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long sub_x2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

}  // namespace vcpcu
