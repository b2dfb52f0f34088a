/*
 * ozaki_model.c -- host model of the Ozaki-form interval product.
 *
 * TEST INFRASTRUCTURE ONLY (see vcp_oracle.c).  The GPU form must be
 * bit-identical to this model, which restates, in plain C and integer
 * arithmetic, the same slicing, summation order and directed-rounding
 * reassembly:
 *
 *  - operands: kv-style midrad of every interval entry (as pidblas_assist::
 *    midrad, vcp/pidblas.hpp:43-51), P = |mA| +ru rA, S = |mB|;
 *  - exponents: E with max |x| <= 2^(E-1) per row (left) / column (right);
 *    the reference's per-row/column sigma = 2^(e+s) split of
 *    pddblas_assist::split_row/split_col (vcp/pddblas.hpp:82-154);
 *  - digits: N = x 2^(8s-E) rounded (nearest-even; upward for the radius
 *    factors) and written as s balanced base-256 digits in [-128, 128];
 *  - products: pairs (p, q) with p + q <= s + 1 (midpoint; for the radius
 *    factors all pairs, or p + q <= 3 in the CRT form with the fast-radius
 *    flag and sr = 2: the pair of the two low digits left out) in ascending
 *    t = p + q, each split into chunks of
 *    1024 inner indices; chunk sums are folded into the int64 value
 *    W = sum C_t 2^(8 (t_ref - t)) every 64 chunks and at the end of each
 *    t (right shifts floor) -- the accumulation order of the reference's
 *    ozaki_acc (vcp/pddblas.hpp:160-193: t ascending, p ascending);
 *  - reassembly: [RD(W u) - e, RU((W + R) u) + e] with u = 2^(E + F - 8 t_ref),
 *    e = RU(trunc + T), trunc = 2^(E-8s) RU(RU(0.515625 delta) 2^(F-8) +
 *    RU(beta/2)), T = RU(RU((S'+R') u') + RU((S''+R'') u''));
 *  - radius products: S = RU(chunk 2^(8 (t_ref - t)) + S) in fp32 over the
 *    digit pairs (t ascending, p ascending) and their exact chunk sums, in
 *    order (the slice GEMM epilogue's single-rounding FMA chain, one fold
 *    per product and tile); CRT form with the fast-radius flag (s + 0x100):
 *    the left-out low x low pair,
 *    sum_k lo_A lo_B 2^(8 (t_ref - 4)) with t_ref = 3, is bounded by Cauchy-
 *    Schwarz, b = RU(RU(sqrt(RU(QA_i))) 2^-8 RU(sqrt(RU(QB_j)))) with QA_i,
 *    QB_j the row's / column's sums of squared low digits (RU in fp32), and
 *    S becomes RU(S + b).
 */
#include <fenv.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OZ_ZERO_EXP (-30000)
#define OZ_CHUNK 1024
#define OZ_FOLD 64
#define OZ_MAXS 12

static uint64_t dbits(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
}
static double bitsd(uint64_t b) {
  double x;
  memcpy(&x, &b, 8);
  return x;
}

static int oz_exponent(double amax) {
  uint64_t b = dbits(amax);
  int be = (int)((b >> 52) & 0x7ff);
  uint64_t mant = b & ((1ULL << 52) - 1);
  if (be == 0 && mant == 0) return OZ_ZERO_EXP;
  if (be == 0) {
    int bl = 0;
    while (mant) {
      mant >>= 1;
      ++bl;
    }
    return bl - 1073;
  }
  return be - 1021;
}

static __int128 oz_scaled_int_bits(double x, int E, int bits, int up) {
  uint64_t b = dbits(x);
  int neg = (int)(b >> 63), be = (int)((b >> 52) & 0x7ff);
  uint64_t mant = b & ((1ULL << 52) - 1);
  if (be == 0 && mant == 0) return 0;
  int ex;
  if (be == 0)
    ex = -1074;
  else {
    mant |= 1ULL << 52;
    ex = be - 1075;
  }
  int sh = ex + bits - E;
  unsigned __int128 N;
  if (sh >= 0) {
    N = (unsigned __int128)mant << sh;
  } else {
    int r = -sh;
    uint64_t q;
    int rem_nz, above, at;
    if (r >= 64) {
      q = 0;
      rem_nz = mant != 0;
      above = 0;
      at = 0;
    } else {
      q = mant >> r;
      uint64_t rem = mant & ((1ULL << r) - 1), half = 1ULL << (r - 1);
      rem_nz = rem != 0;
      above = rem > half;
      at = rem == half;
    }
    if (up) {
      if (!neg && rem_nz) q += 1;
    } else if (above || (at && (q & 1))) {
      q += 1;
    }
    N = q;
  }
  return neg ? -(__int128)N : (__int128)N;
}

static __int128 oz_scaled_int(double x, int E, int s, int up) {
  return oz_scaled_int_bits(x, E, 8 * s, up);
}

static void oz_digits(__int128 N, int s, int* d) {
  for (int p = s - 1; p >= 1; --p) {
    int lo = (int)((uint64_t)(N + 128) & 255ULL) - 128;
    d[p] = lo;
    N = (N - lo) >> 8;
  }
  d[0] = (int)N;
}

/* Directed operations.  The operands are read through volatile copies
 * after the mode switch and the result is stored to a volatile before the
 * mode is restored, so the compiler cannot move the arithmetic across the
 * fesetround calls (which -frounding-math alone does not guarantee). */
static double add_dir(double a, double b, int mode) {
  volatile double x = a, y = b;
  fesetround(mode);
  volatile double r = x + y;
  fesetround(FE_TONEAREST);
  return r;
}
static double sub_dir(double a, double b, int mode) {
  volatile double x = a, y = b;
  fesetround(mode);
  volatile double r = x - y;
  fesetround(FE_TONEAREST);
  return r;
}
static double mul_dir(double a, double b, int up) {
  volatile double x = a, y = b;
  fesetround(up ? FE_UPWARD : FE_DOWNWARD);
  volatile double r = x * y;
  fesetround(FE_TONEAREST);
  return r;
}
static double fma_ru(double a, double b, double c) {
  volatile double x = a, y = b, z = c;
  fesetround(FE_UPWARD);
  volatile double r = fma(x, y, z);
  fesetround(FE_TONEAREST);
  return r;
}
static double ll2d(long long v, int up) {
  volatile long long x = v;
  fesetround(up ? FE_UPWARD : FE_DOWNWARD);
  volatile double r = (double)x;
  fesetround(FE_TONEAREST);
  return r;
}

/* midrad as in the plain form; the caller runs in round-to-nearest */
static void midrad_rp(double lo, double up, double* m, double* r, double* pabs) {
  double s = lo + up;
  double mm = isfinite(s) ? s * 0.5 : lo * 0.5 + up * 0.5;
  double rr = fmax(sub_dir(mm, lo, FE_UPWARD), sub_dir(up, mm, FE_UPWARD));
  *pabs = add_dir(fabs(mm), rr, FE_UPWARD);
  *m = mm;
  *r = rr;
}

static double scale_dir(double x, int e, int up) {
  while (e > 1023) {
    x = mul_dir(x, 0x1p1023, up);
    e -= 1023;
  }
  while (e < -1022) {
    x = mul_dir(x, 0x1p-1022, up);
    e += 1022;
  }
  return mul_dir(x, bitsd((uint64_t)(e + 1023) << 52), up);
}

static double pow2_ru(int e) {
  if (e >= -1022) return scale_dir(1.0, e, 1);
  if (e >= -1074) return bitsd(1ULL << (e + 1074));
  return bitsd(1ULL);
}

typedef struct {
  int npairs, ngroups;
  int pa[80], pb[80];
  int gstart[27], gt[26];
} pairlist;

static void build_pairs(int sa, int sb, int triangular, pairlist* pl) {
  memset(pl, 0, sizeof(*pl));
  int tmax = triangular ? (sa > sb ? sa : sb) + 1 : sa + sb;
  int n = 0, g = 0;
  for (int t = 2; t <= tmax; ++t) {
    int start = n;
    for (int p = 1; p < t; ++p) {
      int q = t - p;
      if (p > sa || q > sb) continue;
      pl->pa[n] = p - 1;
      pl->pb[n] = q - 1;
      ++n;
    }
    if (n > start) {
      pl->gstart[g] = start;
      pl->gt[g] = t;
      ++g;
    }
  }
  pl->gstart[g] = n;
  pl->npairs = n;
  pl->ngroups = g;
}

static void choose_scaling(const pairlist* pl, int nchunks, int* t_ref, int* R) {
  int best = 2, tmax = pl->gt[pl->ngroups - 1];
  for (int tr = 2; tr <= tmax; ++tr) {
    double bound = 0.0;
    for (int g = 0; g < pl->ngroups; ++g) {
      double np = (double)(pl->gstart[g + 1] - pl->gstart[g]);
      bound += np * nchunks * 16777216.0 * ldexp(1.0, 8 * (tr - pl->gt[g])) + 64.0;
    }
    if (bound < ldexp(1.0, 62)) best = tr;
  }
  int r = 0;
  for (int g = 0; g < pl->ngroups; ++g) {
    if (pl->gt[g] <= best) continue;
    int total = (pl->gstart[g + 1] - pl->gstart[g]) * nchunks;
    r += (total + OZ_FOLD - 1) / OZ_FOLD;
  }
  *t_ref = best;
  *R = r;
}

static long long shift_t(long long c, int sh) { return sh >= 0 ? (c << sh) : (c >> (-sh)); }

/* RU(v) as a float for an integer |v| < 2^62 (the rounding mode is nearest
   here): the nearest float, moved up one unit if it lies below v (the
   comparison is exact: the float is an integer). */
static float i64_to_float_ru(long long v) {
  float f = (float)v;
  if ((long long)f < v) f = nextafterf(f, INFINITY);
  return f;
}

/* fp32 operations rounded upward (operands and result through volatiles, as
   for the double ones) */
static float fadd_ru(float a, float b) {
  volatile float x = a, y = b;
  fesetround(FE_UPWARD);
  volatile float r = x + y;
  fesetround(FE_TONEAREST);
  return r;
}
static float fmul_ru(float a, float b) {
  volatile float x = a, y = b;
  fesetround(FE_UPWARD);
  volatile float r = x * y;
  fesetround(FE_TONEAREST);
  return r;
}
/* RU(sqrt(RU(Q))) scale for a sum Q >= 0 of squared digits (0 for Q = 0),
   scale a power of two (exact) */
static float lowpair_root(long long Q, float scale) {
  if (Q == 0) return 0.0f;
  volatile float q = i64_to_float_ru(Q);
  fesetround(FE_UPWARD);
  volatile float r = sqrtf(q);
  fesetround(FE_TONEAREST);
  return r * scale;
}

/* CRT form: integer bits w per operand for precision parameter s (w = 7 s,
 * lowered while 16 moduli cannot hold K 2^(2w-1)); the moduli are those of
 * the GPU form (pairwise coprime, <= 256). */
static const int OZ_MOD[16] = {256, 255, 253, 251, 247, 241, 239, 233,
                               229, 227, 223, 217, 211, 199, 197, 193};
static int crt_bits(int K, int s) {
  int w = 7 * s;
  if (w > 62) w = 62; /* |A'|, |B'| <= 2^61 stay 64-bit integers */
  const int Keff = K > 1 ? K : 1;
  for (;;) {
    double need = 2.0 * w + log2((double)Keff) + 0.01, bits = 0.0;
    int L = 0;
    while (L < 16 && bits <= need) bits += log2((double)OZ_MOD[L++]);
    if (bits > need) return w;
    --w;
  }
}

/* RD and RU of (-1)^neg * mag * 2^e for an unsigned 128-bit mag, the same
 * two steps as the GPU: the top 64 bits with a sticky bit, converted in the
 * direction, then scaled in the direction. */
static void big_to_dir(unsigned __int128 mag, int neg, int e, double* lo, double* up) {
  if (mag == 0) {
    *lo = *up = 0.0;
    return;
  }
  int bl = 0;
  for (unsigned __int128 t = mag; t; t >>= 1) ++bl;
  unsigned long long t;
  int sh = 0;
  if (bl <= 64) {
    t = (unsigned long long)mag;
  } else {
    sh = bl - 64;
    t = (unsigned long long)(mag >> sh);
    if (mag & ((((unsigned __int128)1) << sh) - 1)) t |= 1ULL;
  }
  volatile unsigned long long vt = t;
  fesetround(FE_DOWNWARD);
  volatile double a_dn = (double)vt;
  fesetround(FE_UPWARD);
  volatile double a_up = (double)vt;
  fesetround(FE_TONEAREST);
  if (!neg) {
    *lo = scale_dir(a_dn, e + sh, 0);
    *up = scale_dir(a_up, e + sh, 1);
  } else {
    *lo = -scale_dir(a_up, e + sh, 1);
    *up = -scale_dir(a_dn, e + sh, 0);
  }
}

/*
 * The whole Ozaki-form product: C (m x n, kv layout, ld m) = [A] (m x k) *
 * [B] (k x n), precision s, sr radius slices.  crt == 0: the midpoint is the
 * triangular sum of s digit slices; crt != 0: the midpoint is the exact
 * product of w-bit integers (what the GPU recovers from its residues).
 * Digits (in [-128, 128]) are kept as int16.  Returns 0, or 3 on non-finite
 * input (result NaN).
 */
static int ozaki_model(int m, int n, int k, const double* A, const double* B, double* Cout,
                       int s, int sr, int crt) {
  /* s + 0x100: fast radius products (CRT form: the low x low digit pair left
     out and bounded) */
  const int fast_rad = (s & 0x100) != 0;
  s &= ~0x100;
  if (s <= 0) s = 8;
  const int lowb = crt && fast_rad; /* the low x low radius pair left out and bounded */
  if (lowb && sr != 2) return 2;      /* the bound is written for sr = 2 */
  const int prev = fegetround();
  fesetround(FE_TONEAREST);
  const int Kp = k <= 0 ? 64 : (k + 63) / 64 * 64;
  const int nchunks = (Kp + OZ_CHUNK - 1) / OZ_CHUNK;
  int nonfinite = 0;
  /* --- left factor ---------------------------------------------------- */
  double* mA = calloc((size_t)m * (k > 0 ? k : 1), sizeof(double));
  double* rA = calloc((size_t)m * (k > 0 ? k : 1), sizeof(double));
  double* pA = calloc((size_t)m * (k > 0 ? k : 1), sizeof(double));
  for (long t = 0; t < (long)m * k; ++t) {
    double lo = A[2 * t], up = A[2 * t + 1];
    if (!isfinite(lo) || !isfinite(up)) {
      nonfinite = 1;
      continue;
    }
    midrad_rp(lo, up, &mA[t], &rA[t], &pA[t]);
  }
  int* Em = malloc(sizeof(int) * m);
  int* Ep = malloc(sizeof(int) * m);
  int* Er = malloc(sizeof(int) * m);
  long long* delta = calloc(m, sizeof(long long));
  long long* QA = calloc(2 * (size_t)m, sizeof(long long)); /* sum_k lo^2: P, rA per row */
  /* digits stored as int16 in [-128, 128]: planes [p][i][Kp] */
  int16_t* dAm = calloc((size_t)s * m * Kp, sizeof(int16_t));
  int16_t* dAp = calloc((size_t)sr * m * Kp, sizeof(int16_t));
  int16_t* dAr = calloc((size_t)sr * m * Kp, sizeof(int16_t));
  for (int i = 0; i < m; ++i) {
    double am = 0, ap = 0, ar = 0;
    for (int p = 0; p < k; ++p) {
      long t = i + (long)p * m;
      am = fmax(am, fabs(mA[t]));
      ap = fmax(ap, pA[t]);
      ar = fmax(ar, rA[t]);
    }
    Em[i] = oz_exponent(am);
    Ep[i] = oz_exponent(ap);
    Er[i] = oz_exponent(ar);
    int d[OZ_MAXS];
    for (int p = 0; p < k; ++p) {
      long t = i + (long)p * m;
      if (!crt && Em[i] != OZ_ZERO_EXP && mA[t] != 0.0) {
        oz_digits(oz_scaled_int(mA[t], Em[i], s, 0), s, d);
        for (int q = 0; q < s; ++q) {
          dAm[((size_t)q * m + i) * Kp + p] = (int16_t)d[q];
          delta[i] += abs(d[q]);
        }
      }
      if (Ep[i] != OZ_ZERO_EXP && pA[t] != 0.0) {
        oz_digits(oz_scaled_int(pA[t], Ep[i], sr, 1), sr, d);
        for (int q = 0; q < sr; ++q) dAp[((size_t)q * m + i) * Kp + p] = (int16_t)d[q];
        QA[2 * i] += (long long)d[sr - 1] * d[sr - 1];
      }
      if (Er[i] != OZ_ZERO_EXP && rA[t] != 0.0) {
        oz_digits(oz_scaled_int(rA[t], Er[i], sr, 1), sr, d);
        for (int q = 0; q < sr; ++q) dAr[((size_t)q * m + i) * Kp + p] = (int16_t)d[q];
        QA[2 * i + 1] += (long long)d[sr - 1] * d[sr - 1];
      }
    }
  }
  const int wbits = crt ? crt_bits(k, s) : 0;
  long long* Ai = NULL;      /* A' (m x k, row-major per row i) */
  unsigned long long* Ahi = NULL, *Alo = NULL;
  long long* Bi = NULL;      /* B' (column j contiguous) */
  if (crt) {
    const int kk1 = k > 0 ? k : 1;
    Ai = calloc((size_t)m * kk1, sizeof(long long));
    Ahi = calloc(m, sizeof(unsigned long long));
    Alo = calloc(m, sizeof(unsigned long long));
    Bi = calloc((size_t)n * kk1, sizeof(long long));
    for (int i = 0; i < m; ++i)
      for (int p = 0; p < k; ++p) {
        const double x = mA[i + (long)p * m];
        long long a = (Em[i] == OZ_ZERO_EXP || x == 0.0)
                          ? 0 : (long long)oz_scaled_int_bits(x, Em[i], wbits, 0);
        Ai[(size_t)i * kk1 + p] = a;
        unsigned long long ua = (unsigned long long)(a < 0 ? -a : a);
        Ahi[i] += ua >> 32;
        Alo[i] += ua & 0xffffffffULL;
      }
  }
  /* --- right factor --------------------------------------------------- */
  int* Fm = malloc(sizeof(int) * n);
  int* Fr = malloc(sizeof(int) * n);
  double* beta = malloc(sizeof(double) * n);
  int16_t* dBm = calloc((size_t)s * n * Kp, sizeof(int16_t));
  int16_t* dBr = calloc((size_t)sr * n * Kp, sizeof(int16_t));
  int16_t* dBs = calloc((size_t)sr * n * Kp, sizeof(int16_t));
  long long* QB = calloc(2 * (size_t)n, sizeof(long long)); /* sum_k lo^2: rB, |mB| per column */
  double* mcol = malloc(sizeof(double) * (k > 0 ? k : 1));
  double* rcol = malloc(sizeof(double) * (k > 0 ? k : 1));
  for (int j = 0; j < n; ++j) {
    double am = 0, ar = 0;
    double part[256];
    for (int t = 0; t < 256; ++t) part[t] = 0.0;
    for (int p = 0; p < k; ++p) {
      long t = p + (long)j * k;
      double lo = B[2 * t], up = B[2 * t + 1], pp;
      if (!isfinite(lo) || !isfinite(up)) {
        nonfinite = 1;
        mcol[p] = rcol[p] = 0.0;
        continue;
      }
      midrad_rp(lo, up, &mcol[p], &rcol[p], &pp);
      am = fmax(am, fabs(mcol[p]));
      ar = fmax(ar, rcol[p]);
      part[p % 256] = add_dir(part[p % 256], fabs(mcol[p]), FE_UPWARD);
    }
    for (int w = 128; w > 0; w >>= 1)
      for (int t = 0; t < w; ++t) part[t] = add_dir(part[t], part[t + w], FE_UPWARD);
    beta[j] = part[0];
    Fm[j] = oz_exponent(am);
    Fr[j] = oz_exponent(ar);
    int d[OZ_MAXS];
    uint64_t bhi = 0, blo = 0;
    for (int p = 0; p < k; ++p) {
      if (Fm[j] != OZ_ZERO_EXP && mcol[p] != 0.0) {
        if (!crt) {
          oz_digits(oz_scaled_int(mcol[p], Fm[j], s, 0), s, d);
          for (int q = 0; q < s; ++q) dBm[((size_t)q * n + j) * Kp + p] = (int16_t)d[q];
        } else {
          const long long bi = (long long)oz_scaled_int_bits(mcol[p], Fm[j], wbits, 0);
          Bi[(size_t)j * (k > 0 ? k : 1) + p] = bi;
          const uint64_t ub = (uint64_t)(bi < 0 ? -bi : bi);
          bhi += ub >> 32;
          blo += ub & 0xffffffffULL;
        }
        oz_digits(oz_scaled_int(fabs(mcol[p]), Fm[j], sr, 1), sr, d);
        for (int q = 0; q < sr; ++q) dBs[((size_t)q * n + j) * Kp + p] = (int16_t)d[q];
        QB[2 * j + 1] += (long long)d[sr - 1] * d[sr - 1];
      }
      if (Fr[j] != OZ_ZERO_EXP && rcol[p] != 0.0) {
        oz_digits(oz_scaled_int(rcol[p], Fr[j], sr, 1), sr, d);
        for (int q = 0; q < sr; ++q) dBr[((size_t)q * n + j) * Kp + p] = (int16_t)d[q];
        QB[2 * j] += (long long)d[sr - 1] * d[sr - 1];
      }
    }
    /* CRT form: beta_j = RU((sum_k |B'| + ceil(K/2)) 2^(F - w)) >= sum_k |mB|,
       since |mB| 2^(w - F) <= |B'| + 1/2 */
    if (crt)
      beta[j] = Fm[j] == OZ_ZERO_EXP
                    ? 0.0
                    : scale_dir(fma_ru((double)bhi, 0x1p32, (double)(blo + (uint64_t)(k + 1) / 2)),
                                Fm[j] - wbits, 1);
  }
  pairlist pm, pr;
  build_pairs(s, s, 1, &pm);
  build_pairs(sr, sr, lowb, &pr);
  int tm, Rm, trr, Rr;
  choose_scaling(&pm, nchunks, &tm, &Rm);
  choose_scaling(&pr, nchunks, &trr, &Rr);
  int status = nonfinite ? 3 : 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int j = 0; j < n; ++j) {
    fesetround(FE_TONEAREST);
    for (int i = 0; i < m; ++i) {
      /* element W with int16 digits */
      long long W[3];
      const pairlist* pls[3] = {&pr, &pr, &pm};
      const int trefs[3] = {trr, trr, tm};
      const int16_t* as[3] = {dAp, dAr, dAm};
      const int16_t* bs[3] = {dBr, dBs, dBm};
      float Sr[2] = {0.0f, 0.0f}; /* radius products: fp32 upward sums of the folds */
      for (int w = 0; w < 3; ++w) {
        const pairlist* pl = pls[w];
        long long acc = 0;
        int have = 0;
        for (int g = 0; g < pl->ngroups; ++g) {
          int sh = 8 * (trefs[w] - pl->gt[g]);
          long long C = 0;
          int cnt = 0, total = (pl->gstart[g + 1] - pl->gstart[g]) * nchunks, idx = 0;
          for (int pi = pl->gstart[g]; pi < pl->gstart[g + 1]; ++pi) {
            const int16_t* a = as[w] + ((size_t)pl->pa[pi] * m + i) * Kp;
            const int16_t* b = bs[w] + ((size_t)pl->pb[pi] * n + j) * Kp;
            for (int ch = 0; ch < nchunks; ++ch, ++idx) {
              int k0 = ch * OZ_CHUNK, k1 = k0 + OZ_CHUNK < Kp ? k0 + OZ_CHUNK : Kp;
              int s32 = 0;
              for (int kk = k0; kk < k1; ++kk) s32 += (int)a[kk] * (int)b[kk];
              if (w < 2) {
                /* radius products: S = RU(chunk 2^sh + S) over the pairs (t
                   ascending, p ascending) and their chunks, in fp32 -- the
                   slice GEMM's epilogue (sh >= 0: exact integers below 2^53
                   before the one rounding) */
                Sr[w] = i64_to_float_ru((long long)s32 * (1LL << sh) + (long long)Sr[w]);
                continue;
              }
              C += s32;
              ++cnt;
              if (cnt == OZ_FOLD || idx == total - 1) {
                long long v = shift_t(C, sh);
                acc = have ? acc + v : v;
                have = 1;
                C = 0;
                cnt = 0;
              }
            }
          }
        }
        W[w] = acc;
      }
      /* radius bound: RU((S + R) 2^ex) per product (S + R >= 0), RU sum */
      double T = 0.0;
      {
        double bb[2] = {0.0, 0.0};
        const int zz[2] = {Ep[i] == OZ_ZERO_EXP || Fr[j] == OZ_ZERO_EXP,
                           Er[i] == OZ_ZERO_EXP || Fm[j] == OZ_ZERO_EXP};
        const int ex[2] = {Ep[i] + Fr[j] - 8 * trr, Er[i] + Fm[j] - 8 * trr};
        for (int w = 0; w < 2; ++w) {
          if (zz[w]) continue;
          float sv = Rr ? i64_to_float_ru((long long)Sr[w] + Rr) : Sr[w];
          if (lowb) /* the left-out low x low pair */
            sv = fadd_ru(sv, fmul_ru(lowpair_root(QA[2 * i + w], 0x1p-8f),
                                     lowpair_root(QB[2 * j + w], 1.0f)));
          if (sv > 0.0f) bb[w] = scale_dir((double)sv, ex[w], 1);
        }
        T = add_dir(bb[0], bb[1], FE_UPWARD);
      }
      double mlo = 0.0, mup = 0.0, tr = 0.0;
      int z = Em[i] == OZ_ZERO_EXP || Fm[j] == OZ_ZERO_EXP;
      if (!z && crt) {
        const int kk1 = k > 0 ? k : 1;
        __int128 X = 0;
        for (int p = 0; p < k; ++p)
          X += (__int128)Ai[(size_t)i * kk1 + p] * (__int128)Bi[(size_t)j * kk1 + p];
        int neg = X < 0;
        unsigned __int128 mag = (unsigned __int128)(neg ? -X : X);
        big_to_dir(mag, neg, Em[i] + Fm[j] - 2 * wbits, &mlo, &mup);
        double sA = fma_ru((double)Ahi[i], 0x1p32, (double)Alo[i]);
        double t1 = scale_dir(beta[j], Em[i] - wbits - 1, 1);
        double t2 = scale_dir(sA, Em[i] + Fm[j] - 2 * wbits - 1, 1);
        tr = add_dir(t1, t2, FE_UPWARD);
      } else if (!z) {
        int ex = Em[i] + Fm[j] - 8 * tm;
        mlo = scale_dir(ll2d(W[2], 0), ex, 0);
        mup = scale_dir(ll2d(W[2] + Rm, 1), ex, 1);
        double dlt = mul_dir((double)delta[i], 0.515625, 1);
        double bh = mul_dir(beta[j], 0.5, 1);
        double f2 = pow2_ru(Fm[j] - 8);
        double x = fma_ru(dlt, f2, bh);
        tr = scale_dir(x, Em[i] - 8 * s, 1);
      }
      double err = add_dir(tr, T, FE_UPWARD);
      double up = add_dir(mup, err, FE_UPWARD);
      double lo = sub_dir(mlo, err, FE_DOWNWARD);
      if (nonfinite) lo = up = NAN;
      Cout[2 * ((size_t)i + (size_t)j * m)] = lo;
      Cout[2 * ((size_t)i + (size_t)j * m) + 1] = up;
    }
  }
  free(mA); free(rA); free(pA); free(Em); free(Ep); free(Er); free(delta); free(QA); free(QB);
  free(dAm); free(dAp); free(dAr); free(Fm); free(Fr); free(beta);
  free(dBm); free(dBr); free(dBs); free(mcol); free(rcol);
  free(Ai); free(Ahi); free(Alo); free(Bi);
  fesetround(prev);
  return status;
}

/* Slice form (GPU form VCPCU_FORM_OZAKI_SLICES). */
int orc_ozaki_igemm(int m, int n, int k, const double* A, const double* B, double* Cout, int s,
                    int sr) {
  return ozaki_model(m, n, k, A, B, Cout, s, sr, 0);
}

/* CRT form (GPU form VCPCU_FORM_OZAKI). */
int orc_ozaki2_igemm(int m, int n, int k, const double* A, const double* B, double* Cout, int s,
                     int sr) {
  return ozaki_model(m, n, k, A, B, Cout, s, sr, 1);
}

int orc_ozaki_model_version(void) { return 4; }
