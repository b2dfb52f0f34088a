// Bit-exactness check of the integer-pipe binary64 helpers (swfp.cuh)
// against the FP64 instructions they stand in for, on seeded random bit
// patterns of every class: normal operands with exponent gaps from 0 to 70,
// exact and near cancellations, signed zeros, subnormals and operands near
// overflow.  Built and run by tests/test_gpu_swfp.py; prints one line per
// function with its mismatch count.
#include <cstdio>
#include <cuda_runtime.h>

#include "swfp.cuh"

using namespace vcpcu;

__device__ unsigned long long mix(unsigned long long z) {  // splitmix64 finaliser
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// A finite double of class `c` from random bits r (and a partner p for the
// classes built relative to another operand).
__device__ double make(unsigned long long r, int c, double p) {
  const unsigned long long sg = (r >> 63) << 63, mant = r & ((1ULL << 52) - 1);
  const int pe = (int)((sw_bits(p) >> 52) & 0x7ff);
  switch (c) {
    case 0: {  // normal, exponent within 70 of the partner's
      int e = pe + (int)((r >> 52) % 141) - 70;
      e = e < 1 ? 1 : (e > 2046 ? 2046 : e);
      return sw_double(sg | ((unsigned long long)e << 52) | mant);
    }
    case 1:  // the negated partner
      return sw_neg(p);
    case 2: {  // the partner +- a few units of the last place, either sign
      const long long k = (long long)((r >> 52) % 9) - 4;
      const unsigned long long b = sw_bits(p) + (unsigned long long)k;
      return sw_double((b & ~(1ULL << 63)) | sg);
    }
    case 3:  // a signed zero
      return sw_double(sg);
    case 4:  // subnormal
      return sw_double(sg | mant);
    case 5: {  // near overflow
      const int e = 2044 + (int)((r >> 52) % 3);
      return sw_double(sg | ((unsigned long long)e << 52) | mant);
    }
    default: {  // any normal
      const int e = 1 + (int)((r >> 52) % 2046);
      return sw_double(sg | ((unsigned long long)e << 52) | mant);
    }
  }
}

__global__ void check(long n, unsigned long long seed, unsigned long long* bad) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const unsigned long long r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1));
    const int ca = (int)(r1 % 16) < 12 ? 6 : (int)(r1 % 16) - 12 + 3;  // mostly normal
    const double a = make(r1 * 0x2545F4914F6CDD1DULL, ca, 1.0);
    const int cb = (int)(r2 % 10) < 4 ? 0 : (int)(r2 % 10) - 3;  // classes 0..6, 0 most often
    const double b = make(r2 * 0x2545F4914F6CDD1DULL, cb, a);
    // sign flip
    if (sw_bits(sw_neg(a)) != sw_bits(-a)) atomicAdd(&bad[0], 1ULL);
    // kv midrad of [min, max]
    const bool lt = __dsub_rn(a, b) < 0.0;
    const double lo = lt ? a : b, hi = lt ? b : a;
    double m1, r1d, p1, m2, r2d, p2;
    sw_midrad(lo, hi, m1, r1d, p1);
    sw_midrad_hw(lo, hi, m2, r2d, p2);
    if (sw_bits(m1) != sw_bits(m2) || sw_bits(r1d) != sw_bits(r2d) || sw_bits(p1) != sw_bits(p2))
      atomicAdd(&bad[1], 1ULL);
  }
}

int main() {
  unsigned long long* bad = nullptr;
  if (cudaMalloc(&bad, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
  cudaMemset(bad, 0, 2 * sizeof(unsigned long long));
  const long n = 1L << 24;
  for (unsigned long long seed = 1; seed <= 4; ++seed) check<<<152 * 16, 256>>>(n, seed * 0x9E37ULL, bad);
  unsigned long long h[2] = {0, 0};
  if (cudaMemcpy(h, bad, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  printf("cases %ld\n", 4 * n);
  printf("sw_neg mismatches %llu\n", h[0]);
  printf("sw_midrad mismatches %llu\n", h[1]);
  return 0;
}
