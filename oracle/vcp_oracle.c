/*
 * vcp_oracle.c -- CPU oracle for the verified GEMM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this code, and only as
 * the checker or the timed CPU baseline; the GPU product never calls it.
 *
 * Contents (each restating the reference's own definition):
 *   orc_rmatmul / orc_udmatmul
 *       vblas rmatmul / udmatmul (vblas/rmatmul.hpp:102, vblas/udmatmul.hpp:758):
 *       every C entry is the ascending sequential FMA chain over the inner
 *       index, rounded in the requested direction, starting from +0.0
 *       (vblas/README.md "packing layout"; micro-kernel
 *       vblas/rmatmul_avx512.hpp:195-242 continues the chain through C).
 *       m <= 0 or k <= 0: no-op; n <= 0: C zeroed (rmatmul_avx512.hpp:482-490).
 *       Portable C with per-thread fesetround + fma(), OpenMP over column
 *       blocks, the same scheme as the NEON / no-SIMD backends
 *       (vblas/rmatmul_neon.hpp, vblas/rmatmul_nosimd.hpp).
 *   orc_midrad
 *       kv-style midpoint/radius used by pidblas_assist::midrad
 *       (vcp/pidblas.hpp:43-51): m = RN((lo+up)/2) (halves first if lo+up
 *       overflows), r = max(RU(m-lo), RU(up-m)).
 *   orc_pidblas_mulmm
 *       pidblas::mulmm (vcp/pidblas.hpp:239-294) with orc_rmatmul as its
 *       dgemm_, in the reference's exact operation order.
 *   orc_ilss_verify
 *       the verification of imats::linearsolve (vcp/imats.hpp:293-364) for a
 *       given approximate inverse R and solution mx, step by step with the
 *       reference's pidblas products and kv interval operations.
 *   orc_exact_hull / orc_exact_dot
 *       exact long-accumulator dot products (a Kulisch-style fixed-point
 *       accumulator over the whole binary64 product range) rounded down/up
 *       to double: the containment oracle.
 *
 * Build: gcc -O3 -fopenmp -frounding-math -ffp-contract=off (see build.py).
 */
#include <fenv.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#pragma STDC FENV_ACCESS ON

static int fe_mode(int rnd) {
  if (rnd == 1) return FE_UPWARD;
  if (rnd == -1) return FE_DOWNWARD;
  return FE_TONEAREST;
}

/* ---------------------------------------------------------------------------
 * Directed-rounding GEMM (vblas naming: A m x n, B n x k, C m x k).
 * Blocking: column blocks of NR=4 C columns are distributed over threads;
 * inside, row blocks of MR=8 and inner blocks of KC keep the A panel hot.
 * The chain of each C entry runs over the inner index in ascending order,
 * continuing through C between inner blocks, so blocking never changes it.
 * ------------------------------------------------------------------------- */
#define ORC_MR 8
#define ORC_NR 4
#define ORC_KC 256
#define ORC_MC 512

#if defined(__aarch64__)
#include <arm_neon.h>
/* Full 8 x 4 tile with NEON: every lane runs one entry's chain, each step a
 * fused multiply-add rounded in the current (FPCR) rounding mode -- the same
 * operation, in the same order, as the scalar fma() below, so the bits do
 * not change (the reference's vblas/rmatmul_neon.hpp organises its tiles the
 * same way).  16 accumulator registers, 4 for A, 4 broadcast B values. */
static void micro_chain_8x4_neon(int kc, const double* A, long lda, const double* B, long ldb,
                                 double* C, long ldc, int first) {
  float64x2_t c0[4], c1[4], c2[4], c3[4];
  for (int r = 0; r < 4; ++r) {
    if (first) {
      c0[r] = c1[r] = c2[r] = c3[r] = vdupq_n_f64(0.0);
    } else {
      c0[r] = vld1q_f64(C + 2 * r);
      c1[r] = vld1q_f64(C + ldc + 2 * r);
      c2[r] = vld1q_f64(C + 2 * ldc + 2 * r);
      c3[r] = vld1q_f64(C + 3 * ldc + 2 * r);
    }
  }
  const double* b0p = B;
  const double* b1p = B + ldb;
  const double* b2p = B + 2 * ldb;
  const double* b3p = B + 3 * ldb;
  for (int p = 0; p < kc; ++p) {
    const double* ap = A + p * lda;
    const float64x2_t a0 = vld1q_f64(ap), a1 = vld1q_f64(ap + 2), a2 = vld1q_f64(ap + 4),
                      a3 = vld1q_f64(ap + 6);
    const float64x2_t b0 = vdupq_n_f64(b0p[p]), b1 = vdupq_n_f64(b1p[p]),
                      b2 = vdupq_n_f64(b2p[p]), b3 = vdupq_n_f64(b3p[p]);
    c0[0] = vfmaq_f64(c0[0], a0, b0); c0[1] = vfmaq_f64(c0[1], a1, b0);
    c0[2] = vfmaq_f64(c0[2], a2, b0); c0[3] = vfmaq_f64(c0[3], a3, b0);
    c1[0] = vfmaq_f64(c1[0], a0, b1); c1[1] = vfmaq_f64(c1[1], a1, b1);
    c1[2] = vfmaq_f64(c1[2], a2, b1); c1[3] = vfmaq_f64(c1[3], a3, b1);
    c2[0] = vfmaq_f64(c2[0], a0, b2); c2[1] = vfmaq_f64(c2[1], a1, b2);
    c2[2] = vfmaq_f64(c2[2], a2, b2); c2[3] = vfmaq_f64(c2[3], a3, b2);
    c3[0] = vfmaq_f64(c3[0], a0, b3); c3[1] = vfmaq_f64(c3[1], a1, b3);
    c3[2] = vfmaq_f64(c3[2], a2, b3); c3[3] = vfmaq_f64(c3[3], a3, b3);
  }
  for (int r = 0; r < 4; ++r) {
    vst1q_f64(C + 2 * r, c0[r]);
    vst1q_f64(C + ldc + 2 * r, c1[r]);
    vst1q_f64(C + 2 * ldc + 2 * r, c2[r]);
    vst1q_f64(C + 3 * ldc + 2 * r, c3[r]);
  }
}
#endif

static void micro_chain(int mr, int nr, int kc, const double* A, long lda, const double* B,
                        long ldb, double* C, long ldc, int first) {
#if defined(__aarch64__)
  if (mr == ORC_MR && nr == ORC_NR) {
    micro_chain_8x4_neon(kc, A, lda, B, ldb, C, ldc, first);
    return;
  }
#endif
  double acc[ORC_NR][ORC_MR];
  for (int j = 0; j < ORC_NR; ++j)
    for (int i = 0; i < ORC_MR; ++i)
      acc[j][i] = (first || j >= nr || i >= mr) ? 0.0 : C[i + j * ldc];
  if (mr == ORC_MR && nr == ORC_NR) {
    for (int p = 0; p < kc; ++p) {
      const double* ap = A + p * lda;
      const double b0 = B[p], b1 = B[p + ldb], b2 = B[p + 2 * ldb], b3 = B[p + 3 * ldb];
      for (int i = 0; i < ORC_MR; ++i) acc[0][i] = fma(ap[i], b0, acc[0][i]);
      for (int i = 0; i < ORC_MR; ++i) acc[1][i] = fma(ap[i], b1, acc[1][i]);
      for (int i = 0; i < ORC_MR; ++i) acc[2][i] = fma(ap[i], b2, acc[2][i]);
      for (int i = 0; i < ORC_MR; ++i) acc[3][i] = fma(ap[i], b3, acc[3][i]);
    }
  } else {
    for (int p = 0; p < kc; ++p)
      for (int j = 0; j < nr; ++j) {
        const double b = B[p + j * ldb];
        for (int i = 0; i < mr; ++i) acc[j][i] = fma(A[i + p * lda], b, acc[j][i]);
      }
  }
  for (int j = 0; j < nr; ++j)
    for (int i = 0; i < mr; ++i) C[i + j * ldc] = acc[j][i];
}

void orc_rmatmul_ld(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                    double* C, long ldc, int rnd, int nthreads) {
  if (m <= 0 || k <= 0) return;
  if (n <= 0) {
    for (long j = 0; j < k; ++j)
      for (long i = 0; i < m; ++i) C[i + j * ldc] = 0.0;
    return;
  }
  const int mode = fe_mode(rnd);
  const int ncb = (k + ORC_NR - 1) / ORC_NR;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    const int prev = fegetround();
    fesetround(mode);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int cb = 0; cb < ncb; ++cb) {
      const int j0 = cb * ORC_NR, nr = (k - j0 < ORC_NR) ? k - j0 : ORC_NR;
      for (int p0 = 0; p0 < n; p0 += ORC_KC) {
        const int kc = (n - p0 < ORC_KC) ? n - p0 : ORC_KC;
        for (int i0 = 0; i0 < m; i0 += ORC_MR) {
          const int mr = (m - i0 < ORC_MR) ? m - i0 : ORC_MR;
          micro_chain(mr, nr, kc, A + i0 + (long)p0 * lda, lda, B + p0 + (long)j0 * ldb, ldb,
                      C + i0 + (long)j0 * ldc, ldc, p0 == 0);
        }
      }
    }
    fesetround(prev);
  }
}

void orc_rmatmul(int m, int n, int k, const double* A, const double* B, double* C, int rnd,
                 int nthreads) {
  orc_rmatmul_ld(m, n, k, A, m, B, n > 0 ? n : 1, C, m, rnd, nthreads);
}

void orc_udmatmul(int m, int n, int k, const double* A, const double* B, double* CU, double* CD,
                  int nthreads) {
  orc_rmatmul(m, n, k, A, B, CU, 1, nthreads);
  orc_rmatmul(m, n, k, A, B, CD, -1, nthreads);
}

/* ---------------------------------------------------------------------------
 * midrad and the pidblas::mulmm restatement.
 * ------------------------------------------------------------------------- */
/* kv layout (pairs {inf,sup}) -> mid / rad planes, count entries.  The
 * midpoints are formed in one round-to-nearest pass, the radii in one
 * round-upward pass. */
/* Elementwise passes run on all threads (each sets its own rounding mode;
 * the results do not depend on the partition). */
void orc_midrad(long count, const double* X, double* mid, double* rad) {
#ifdef _OPENMP
#pragma omp parallel if (count > 65536)
#endif
  {
    const int prev = fegetround();
    fesetround(FE_TONEAREST);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long i = 0; i < count; ++i) {
      const double lo = X[2 * i], up = X[2 * i + 1];
      double s = lo + up;
      mid[i] = isfinite(s) ? s * 0.5 : lo * 0.5 + up * 0.5;
    }
    fesetround(FE_UPWARD);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long i = 0; i < count; ++i) {
      const double lo = X[2 * i], up = X[2 * i + 1];
      rad[i] = fmax(mid[i] - lo, up - mid[i]);
    }
    fesetround(prev);
  }
}

/* pidblas::mulmm, GEMM naming: C (m x n) = A (m x k) * B (k x n); A, B, C in
 * kv layout, column-major with ld = rows.  Order (vcp/pidblas.hpp:256-293):
 *   lC = RD gemm(mA, mB); uC = RU gemm(mA, mB)
 *   mA = |mA| +RU rA; temp = RU gemm(mA, rB); mA2 = RU gemm(rA, |mB|)
 *   temp = temp +RU mA2; uC = uC +RU temp; lC = lC -RD temp.           */
int orc_pidblas_mulmm(int m, int n, int k, const double* A, const double* B, double* C,
                      int nthreads) {
  if (m <= 0 || n <= 0) return 0;
  if (k < 0) k = 0;
  const long na = (long)m * k, nb = (long)k * n, nc = (long)m * n;
  double* buf = (double*)malloc(sizeof(double) * (2 * na + 2 * nb + 4 * nc + 1));
  if (!buf) return 1;
  double *mA = buf, *rA = mA + na, *mB = rA + na, *rB = mB + nb;
  double *lC = rB + nb, *uC = lC + nc, *temp = uC + nc, *t2 = temp + nc;
  const int prev = fegetround();
  orc_midrad(na, A, mA, rA);
  orc_midrad(nb, B, mB, rB);
  orc_rmatmul(m, k, n, mA, mB, lC, -1, nthreads);
  orc_rmatmul(m, k, n, mA, mB, uC, 1, nthreads);
#ifdef _OPENMP
#pragma omp parallel if (na + nb > 65536)
#endif
  {
    const int pv = fegetround();
    fesetround(FE_UPWARD);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long i = 0; i < na; ++i) mA[i] = fabs(mA[i]) + rA[i];
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long i = 0; i < nb; ++i) mB[i] = fabs(mB[i]);
    fesetround(pv);
  }
  orc_rmatmul(m, k, n, mA, rB, temp, 1, nthreads);
  orc_rmatmul(m, k, n, rA, mB, t2, 1, nthreads);
#ifdef _OPENMP
#pragma omp parallel if (nc > 65536)
#endif
  {
    const int pv = fegetround();
    fesetround(FE_UPWARD);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long i = 0; i < nc; ++i) {
      temp[i] = temp[i] + t2[i];
      uC[i] = uC[i] + temp[i];
    }
    fesetround(FE_DOWNWARD);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long i = 0; i < nc; ++i) lC[i] = lC[i] - temp[i];
    fesetround(pv);
  }
  fesetround(prev);
  for (long i = 0; i < nc; ++i) {
    C[2 * i] = lC[i];
    C[2 * i + 1] = uC[i];
  }
  free(buf);
  return 0;
}

/* ---------------------------------------------------------------------------
 * Exact accumulator.  Two's complement fixed point, ACC_WORDS x 64 bits, bit
 * 0 has weight 2^-ACC_BIAS.  Every product of two finite doubles (LSB weight
 * >= 2^-2148, magnitude < 2^2048) and sums of up to 2^60 of them fit.
 * ------------------------------------------------------------------------- */
#define ACC_BIAS 2200
#define ACC_WORDS 70
typedef struct {
  uint64_t w[ACC_WORDS];
  int nonfinite; /* set if an Inf/NaN term was seen */
} orc_acc;

static void acc_zero(orc_acc* a) { memset(a, 0, sizeof(*a)); }

/* Split finite x != 0 into integer mantissa and LSB exponent: x = sgn*mant*2^e. */
static void decompose(double x, int* sgn, uint64_t* mant, int* e) {
  uint64_t b;
  memcpy(&b, &x, 8);
  *sgn = (int)(b >> 63);
  int ex = (int)((b >> 52) & 0x7ff);
  uint64_t f = b & ((1ULL << 52) - 1);
  if (ex == 0) {
    *mant = f;
    *e = -1074;
  } else {
    *mant = f | (1ULL << 52);
    *e = ex - 1075;
  }
}

/* a += (neg ? -1 : 1) * (hi:lo) * 2^pos, pos >= 0 the bit position. */
static void acc_add_u128(orc_acc* a, unsigned __int128 v, int pos, int neg) {
  if (v == 0) return;
  int w = pos >> 6, b = pos & 63;
  uint64_t parts[3];
  uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
  if (b == 0) {
    parts[0] = lo;
    parts[1] = hi;
    parts[2] = 0;
  } else {
    parts[0] = lo << b;
    parts[1] = (hi << b) | (lo >> (64 - b));
    parts[2] = hi >> (64 - b);
  }
  if (!neg) {
    unsigned __int128 carry = 0;
    int i = 0;
    for (; i < 3 && w + i < ACC_WORDS; ++i) {
      unsigned __int128 s = (unsigned __int128)a->w[w + i] + parts[i] + carry;
      a->w[w + i] = (uint64_t)s;
      carry = s >> 64;
    }
    for (int j = w + i; carry && j < ACC_WORDS; ++j) {
      unsigned __int128 s = (unsigned __int128)a->w[j] + carry;
      a->w[j] = (uint64_t)s;
      carry = s >> 64;
    }
  } else {
    uint64_t borrow = 0;
    int i = 0;
    for (; i < 3 && w + i < ACC_WORDS; ++i) {
      uint64_t x = a->w[w + i];
      uint64_t d = x - parts[i] - borrow;
      borrow = (x < parts[i]) || (x - parts[i] < borrow);
      a->w[w + i] = d;
    }
    for (int j = w + i; borrow && j < ACC_WORDS; ++j) {
      uint64_t x = a->w[j];
      a->w[j] = x - 1;
      borrow = (x == 0);
    }
  }
}

/* exact product x*y as (sign, 106-bit magnitude, LSB exponent); 0 if zero */
typedef struct {
  int sgn;
  unsigned __int128 mag;
  int e;
} xprod;

static xprod exact_mul(double x, double y) {
  xprod p = {0, 0, 0};
  if (x == 0.0 || y == 0.0) return p;
  int sx, sy, ex, ey;
  uint64_t mx, my;
  decompose(x, &sx, &mx, &ex);
  decompose(y, &sy, &my, &ey);
  p.sgn = sx ^ sy;
  p.mag = (unsigned __int128)mx * my;
  p.e = ex + ey;
  return p;
}

static int bitlen128(unsigned __int128 v) {
  int n = 0;
  while (v) {
    v >>= 1;
    ++n;
  }
  return n;
}

/* compare exact products: -1, 0, 1 */
static int xcmp(xprod a, xprod b) {
  int za = a.mag == 0, zb = b.mag == 0;
  if (za && zb) return 0;
  if (za) return b.sgn ? 1 : -1;
  if (zb) return a.sgn ? -1 : 1;
  if (a.sgn != b.sgn) return a.sgn ? -1 : 1;
  int la = bitlen128(a.mag), lb = bitlen128(b.mag);
  int ta = a.e + la, tb = b.e + lb;
  int c;
  if (ta != tb)
    c = ta > tb ? 1 : -1;
  else {
    unsigned __int128 xa = a.mag << (128 - la), xb = b.mag << (128 - lb);
    c = xa > xb ? 1 : (xa < xb ? -1 : 0);
  }
  return a.sgn ? -c : c;
}

static void acc_add_xprod(orc_acc* a, xprod p) {
  if (p.mag == 0) return;
  acc_add_u128(a, p.mag, p.e + ACC_BIAS, p.sgn);
}

/* Round the accumulator to double: dir = -1 (down) or +1 (up). */
static double acc_round(const orc_acc* a0, int dir) {
  orc_acc a = *a0;
  int neg = (int)(a.w[ACC_WORDS - 1] >> 63);
  if (neg) { /* magnitude = two's complement negation */
    uint64_t carry = 1;
    for (int i = 0; i < ACC_WORDS; ++i) {
      uint64_t x = ~a.w[i] + carry;
      carry = (carry && x == 0) ? 1 : 0;
      a.w[i] = x;
    }
  }
  int top = -1;
  for (int i = ACC_WORDS - 1; i >= 0 && top < 0; --i)
    if (a.w[i]) top = i * 64 + 63 - __builtin_clzll(a.w[i]);
  if (top < 0) return 0.0; /* exact zero: +0.0 */
  const int min_lsb = ACC_BIAS - 1074;
  int lsb = top - 52;
  if (lsb < min_lsb) lsb = min_lsb;
  uint64_t mant = 0;
  for (int bit = top; bit >= lsb; --bit) mant = (mant << 1) | ((a.w[bit >> 6] >> (bit & 63)) & 1);
  int sticky = 0;
  for (int wi = 0; wi < (lsb >> 6) && !sticky; ++wi) sticky = a.w[wi] != 0;
  if (!sticky && (lsb & 63)) sticky = (a.w[lsb >> 6] & ((1ULL << (lsb & 63)) - 1)) != 0;
  /* magnitude rounding: away from zero if (up and positive) or (down and negative) */
  int away = sticky && ((dir > 0 && !neg) || (dir < 0 && neg));
  if (away) mant += 1;
  int e = lsb - ACC_BIAS;
  /* overflow: beyond DBL_MAX */
  double r;
  if (e + 64 - __builtin_clzll(mant) > 1024) {
    int to_inf = (dir > 0 && !neg) || (dir < 0 && neg);
    r = to_inf ? INFINITY : 1.7976931348623157e308;
  } else {
    r = ldexp((double)mant, e); /* exact: mant <= 2^53 */
  }
  return neg ? -r : r;
}

static int nonfinite2(double x, double y) { return !isfinite(x) || !isfinite(y); }

/* Exact hull of sum_p [A(i,p)] * [B(p,j)] for `count` entries (rows[i], cols[i]);
 * A (m x k), B (k x n) in kv layout with ld = rows.  Outputs RD(lower sum)
 * and RU(upper sum).  Entries with a non-finite term get NaN. */
void orc_exact_hull(int m, int n, int k, const double* A, const double* B, long count,
                    const int* rows, const int* cols, double* out_lo, double* out_up,
                    int nthreads) {
  (void)n;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
  for (long t = 0; t < count; ++t) {
    const int i = rows[t], j = cols[t];
    orc_acc lo, up;
    acc_zero(&lo);
    acc_zero(&up);
    int bad = 0;
    for (int p = 0; p < k; ++p) {
      const double* a = A + 2 * ((long)i + (long)p * m);
      const double* b = B + 2 * ((long)p + (long)j * k);
      if (nonfinite2(a[0], a[1]) || nonfinite2(b[0], b[1])) {
        bad = 1;
        break;
      }
      xprod q[4] = {exact_mul(a[0], b[0]), exact_mul(a[0], b[1]), exact_mul(a[1], b[0]),
                    exact_mul(a[1], b[1])};
      xprod mn = q[0], mx = q[0];
      for (int s = 1; s < 4; ++s) {
        if (xcmp(q[s], mn) < 0) mn = q[s];
        if (xcmp(q[s], mx) > 0) mx = q[s];
      }
      acc_add_xprod(&lo, mn);
      acc_add_xprod(&up, mx);
    }
    if (bad) {
      out_lo[t] = NAN;
      out_up[t] = NAN;
    } else {
      out_lo[t] = acc_round(&lo, -1);
      out_up[t] = acc_round(&up, +1);
    }
  }
}

/* Exact point dot products sum_p A(i,p) B(p,j) (A m x k, B k x n, plain doubles,
 * ld = rows), rounded down and up, for `count` entries. */
void orc_exact_dot(int m, int n, int k, const double* A, const double* B, long count,
                   const int* rows, const int* cols, double* out_dn, double* out_up,
                   int nthreads) {
  (void)n;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
  for (long t = 0; t < count; ++t) {
    const int i = rows[t], j = cols[t];
    orc_acc s;
    acc_zero(&s);
    int bad = 0;
    for (int p = 0; p < k; ++p) {
      double a = A[(long)i + (long)p * m], b = B[(long)p + (long)j * k];
      if (nonfinite2(a, b)) {
        bad = 1;
        break;
      }
      acc_add_xprod(&s, exact_mul(a, b));
    }
    out_dn[t] = bad ? NAN : acc_round(&s, -1);
    out_up[t] = bad ? NAN : acc_round(&s, +1);
  }
}

static void acc_add_double(orc_acc* a, double x, int negate) {
  if (x == 0.0) return;
  int sg, e;
  uint64_t mt;
  decompose(x, &sg, &mt, &e);
  acc_add_u128(a, (unsigned __int128)mt, e + ACC_BIAS, sg ^ negate);
}

/* Error of a dd GEMM result against the exact product (pddblas::mulmm,
 * vcp/pddblas.hpp:318-376, computes C ~ A*B in dd).  A (m x k), B (k x n),
 * C (m x n) are dd matrices as {hi, lo} pairs, ld = rows.  For each sampled
 * entry: S = sum_p (A1 + A2)(B1 + B2) exactly (four double products per
 * term), out_err = RU(|S - (C1 + C2)|) and out_abs = RD(|S|). */
void orc_dd_residual(int m, int n, int k, const double* A, const double* B, const double* C,
                     long count, const int* rows, const int* cols, double* out_err,
                     double* out_abs, int nthreads) {
  (void)n;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
  for (long t = 0; t < count; ++t) {
    const int i = rows[t], j = cols[t];
    orc_acc s;
    acc_zero(&s);
    for (int p = 0; p < k; ++p) {
      const double* a = A + 2 * ((long)i + (long)p * m);
      const double* b = B + 2 * ((long)p + (long)j * k);
      acc_add_xprod(&s, exact_mul(a[0], b[0]));
      acc_add_xprod(&s, exact_mul(a[0], b[1]));
      acc_add_xprod(&s, exact_mul(a[1], b[0]));
      acc_add_xprod(&s, exact_mul(a[1], b[1]));
    }
    const double sd = acc_round(&s, -1), su = acc_round(&s, +1);
    out_abs[t] = (sd > 0.0) ? sd : (su < 0.0 ? -su : 0.0);
    const double* c = C + 2 * ((long)i + (long)j * m);
    acc_add_double(&s, c[0], 1);
    acc_add_double(&s, c[1], 1);
    const double du = acc_round(&s, +1), dd = acc_round(&s, -1);
    out_err[t] = fabs(du) > fabs(dd) ? fabs(du) : fabs(dd);
  }
}

/* Exact sum of a list of doubles, rounded in direction dir (self-test hook). */
double orc_exact_sum(long count, const double* x, int dir) {
  orc_acc s;
  acc_zero(&s);
  for (long i = 0; i < count; ++i) {
    if (x[i] == 0.0) continue;
    int sg, e;
    uint64_t mt;
    decompose(x[i], &sg, &mt, &e);
    acc_add_u128(&s, (unsigned __int128)mt, e + ACC_BIAS, sg);
  }
  return acc_round(&s, dir);
}

/* ---------------------------------------------------------------------------
 * The other pidblas products, restated in the reference's operation order
 * over orc_rmatmul (the sequential-chain dgemm / dsyrk).
 * ------------------------------------------------------------------------- */
static void transpose_d(int rows, int cols, const double* X, double* Xt) {
  for (long j = 0; j < cols; ++j)
    for (long i = 0; i < rows; ++i) Xt[j + i * cols] = X[i + j * rows];
}

/* pidblas::mul_im_m (vcp/pidblas.hpp:90-140): C = [A] B, A m x k interval,
 * B k x n point.  pidblas::mul_m_im (:142-196): C = B [A], B m x k point,
 * A k x n interval.  side 0 / 1 selects which. */
int orc_pidblas_mul_point(int side, int m, int n, int k, const double* L, const double* R,
                          double* C, int nthreads) {
  if (m <= 0 || n <= 0) return 0;
  if (k < 0) k = 0;
  const long nl = (long)m * k, nr = (long)k * n, nc = (long)m * n;
  const long ni = side == 0 ? nl : nr;  /* interval factor entries */
  const long np = side == 0 ? nr : nl;  /* point factor entries */
  double* buf = (double*)malloc(sizeof(double) * (2 * ni + np + 3 * nc + 1));
  if (!buf) return 1;
  double *mid = buf, *rad = mid + ni, *absP = rad + ni;
  double *lC = absP + np, *uC = lC + nc, *temp = uC + nc;
  const int prev = fegetround();
  orc_midrad(ni, side == 0 ? L : R, mid, rad);
  const double* P = side == 0 ? R : L;  /* the point factor */
  for (long t = 0; t < np; ++t) absP[t] = fabs(P[t]);
  if (side == 0) {
    orc_rmatmul(m, k, n, mid, P, lC, -1, nthreads);
    orc_rmatmul(m, k, n, mid, P, uC, 1, nthreads);
    orc_rmatmul(m, k, n, rad, absP, temp, 1, nthreads);
  } else {
    orc_rmatmul(m, k, n, P, mid, lC, -1, nthreads);
    orc_rmatmul(m, k, n, P, mid, uC, 1, nthreads);
    orc_rmatmul(m, k, n, absP, rad, temp, 1, nthreads);
  }
  fesetround(FE_UPWARD);
  for (long i = 0; i < nc; ++i) uC[i] = uC[i] + temp[i];
  fesetround(FE_DOWNWARD);
  for (long i = 0; i < nc; ++i) lC[i] = lC[i] - temp[i];
  fesetround(prev);
  for (long i = 0; i < nc; ++i) {
    C[2 * i] = lC[i];
    C[2 * i + 1] = uC[i];
  }
  free(buf);
  return 0;
}

/* pidblas::mulltmm (vcp/pidblas.hpp:296-358): C (n x n) = [A]^T [A], A k x n. */
int orc_pidblas_mulltmm(int n, int k, const double* A, double* C, int nthreads) {
  if (n <= 0) return 0;
  if (k < 0) k = 0;
  const long na = (long)k * n, nc = (long)n * n;
  double* buf = (double*)malloc(sizeof(double) * (5 * (na + 1) + 4 * nc));
  if (!buf) return 1;
  double *mA = buf, *rA = mA + na + 1, *mAt = rA + na + 1, *aAt = mAt + na + 1, *rAt = aAt + na + 1;
  double *lC = rAt + na + 1, *uC = lC + nc, *temp = uC + nc, *rr = temp + nc;
  const int prev = fegetround();
  orc_midrad(na, A, mA, rA);
  transpose_d(k, n, mA, mAt);
  transpose_d(k, n, rA, rAt);
  for (long t = 0; t < na; ++t) aAt[t] = fabs(mAt[t]);
  orc_rmatmul(n, k, n, mAt, mA, lC, -1, nthreads);   /* dsyrk under RD */
  orc_rmatmul(n, k, n, mAt, mA, uC, 1, nthreads);    /* dsyrk under RU */
  orc_rmatmul(n, k, n, aAt, rA, temp, 1, nthreads);  /* temp = |mA|^T rA */
  orc_rmatmul(n, k, n, rAt, rA, rr, 1, nthreads);    /* rA^T rA */
  fesetround(FE_UPWARD);
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) {
      const double t = temp[j + (long)n * i] + rr[i + (long)n * j];
      temp[i + (long)n * j] = temp[i + (long)n * j] + t;
    }
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) temp[j + (long)n * i] = temp[i + (long)n * j];
  for (long i = 0; i < nc; ++i) uC[i] = uC[i] + temp[i];
  fesetround(FE_DOWNWARD);
  for (long i = 0; i < nc; ++i) lC[i] = lC[i] - temp[i];
  fesetround(prev);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const long s = (i <= j) ? i + (long)n * j : j + (long)n * i;  /* upper triangle */
      C[2 * (i + (long)n * j)] = lC[s];
      C[2 * (i + (long)n * j) + 1] = uC[s];
    }
  free(buf);
  return 0;
}

/* pidblas::vmulmm (vcp/pidblas.hpp:198-236): [RD(A^T A), RU(A^T A)], A k x n point. */
int orc_pidblas_vmulmm(int n, int k, const double* A, double* C, int nthreads) {
  if (n <= 0) return 0;
  if (k < 0) k = 0;
  const long na = (long)k * n, nc = (long)n * n;
  double* buf = (double*)malloc(sizeof(double) * (na + 1 + 2 * nc));
  if (!buf) return 1;
  double *At = buf, *lo = At + na + 1, *up = lo + nc;
  transpose_d(k, n, A, At);
  orc_rmatmul(n, k, n, At, A, lo, -1, nthreads);
  orc_rmatmul(n, k, n, At, A, up, 1, nthreads);
  for (long i = 0; i < nc; ++i) {
    C[2 * i] = lo[i];
    C[2 * i + 1] = up[i];
  }
  free(buf);
  return 0;
}

/* The bound ||R [A] - I||_inf of imats::linearsolve (vcp/imats.hpp:316-336,
 * mats::norminf vcp/mats.hpp:1583-1597). */
double orc_norm_I_minus_RA(int n, const double* R, const double* A, int nthreads) {
  double* b = (double*)malloc(sizeof(double) * 2 * (size_t)n * n);
  if (!b) return NAN;
  orc_pidblas_mul_point(1, n, n, n, R, A, b, nthreads);
  const int prev = fegetround();
  double g = -INFINITY;
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) {
      double lo = b[2 * (i + (long)n * j)], up = b[2 * (i + (long)n * j) + 1];
      if (i == j) {
        volatile double vl = lo, vu = up;
        fesetround(FE_DOWNWARD);
        volatile double l2 = vl - 1.0;
        fesetround(FE_UPWARD);
        volatile double u2 = vu - 1.0;
        fesetround(FE_TONEAREST);
        lo = l2;
        up = u2;
      }
      const double mg = fmax(fabs(lo), fabs(up));
      volatile double vs = s, vm = mg;
      fesetround(FE_UPWARD);
      volatile double ns = (j == 0) ? vm : vs + vm;
      fesetround(FE_TONEAREST);
      s = ns;
    }
    if (isnan(s))
      g = NAN;
    else if (!isnan(g) && s > g)
      g = s;
  }
  fesetround(prev);
  free(b);
  return g;
}

/* ---------------------------------------------------------------------------
 * imats::linearsolve's verification (vcp/imats.hpp:293-364) given its
 * approximate inverse R of mid(A) and approximate solution mx = R mid(b).
 * A n x n, b n x nrhs kv intervals; R, mx point; x n x nrhs kv.  Steps and
 * the kv operations they use (kv interval arithmetic as in the kv stand-in:
 * outward-rounded endpoints, abs, max of upper ends in std::max order):
 *   P = [A] mx        pidblas::mul_im_m                         :305
 *   P = P - [b]       subsmmA, [RD(P.lo - b.up), RU(P.up - b.lo)] :307
 *   r = R P           pidblas::mul_m_im                         :309
 *   E = R [A]         pidblas::mul_m_im; E(i,i) -= 1             :317-326
 *   G = sup ||E||_inf mats::norminf (row sums of sup|E| upward)   :329
 *   t = sup || |r| ||_inf (vector: largest sup|r|; matrix: rows)  :336
 *   g = [t,t] / (1 - [G,G])                                      :341
 *   H = |E| (g ... g) pidblas::mulmm                              :353
 *   x = mx + [-u, u], u = RU(sup|r| + sup H)                       :355-363
 * E_in (kv, n x n), when given, replaces the product R [A] (so that the
 * steps can be checked on the tensor-core form's R [A]).  Returns 0, or 2
 * when G >= 1 (the reference throws vcp::verification_error; x untouched).
 * ------------------------------------------------------------------------- */
static double rnd_op(int mode, double a, double b, char op) {
  volatile double va = a, vb = b;
  const int prev = fegetround();
  fesetround(mode);
  volatile double r = op == '+' ? va + vb : op == '-' ? va - vb : va / vb;
  fesetround(prev);
  return r;
}
static double rnd_op2(int mode, double a, double b) {
  volatile double va = a, vb = b;
  const int prev = fegetround();
  fesetround(mode);
  volatile double r = va * vb;
  fesetround(prev);
  return r;
}
static double kv_abs_sup(double lo, double up) {
  if (lo >= 0.0) return up;
  if (up <= 0.0) return -lo;
  return (-lo < up) ? up : -lo;
}
/* sup of mats::norminf over an interval matrix (rows x cols, kv, ld = rows) */
static double norminf_sup(int rows, int cols, const double* X) {
  const int mat = rows > 1 && cols > 1;
  double c = 0.0;
  if (!mat) {  /* 'S', 'C', 'R': the largest |x| */
    const long cnt = (long)rows * cols;
    c = kv_abs_sup(X[0], X[1]);
    for (long i = 1; i < cnt; ++i) {
      const double a = kv_abs_sup(X[2 * i], X[2 * i + 1]);
      c = (a < c) ? c : a;
    }
    return c;
  }
  for (int i = 0; i < rows; ++i) {
    double s = kv_abs_sup(X[2 * i], X[2 * i + 1]);
    for (int j = 1; j < cols; ++j) {
      const long o = i + (long)j * rows;
      s = rnd_op(FE_UPWARD, s, kv_abs_sup(X[2 * o], X[2 * o + 1]), '+');
    }
    c = (i == 0) ? s : ((s < c) ? c : s);
  }
  return c;
}

int orc_ilss_verify(int n, int nrhs, const double* A, const double* b, const double* R,
                    const double* mx, const double* E_in, double* x, double* bound,
                    int nthreads) {
  const long nv = (long)n * nrhs, nn = (long)n * n;
  double* buf = (double*)malloc(sizeof(double) * (2 * nn + 8 * nv + 2));
  if (!buf) return 1;
  double *E = buf, *P = E + 2 * nn, *r = P + 2 * nv, *T = r + 2 * nv, *H = T + 2 * nv;
  orc_pidblas_mul_point(0, n, nrhs, n, A, mx, P, nthreads);
  for (long i = 0; i < nv; ++i) {
    const double lo = rnd_op(FE_DOWNWARD, P[2 * i], b[2 * i + 1], '-');
    const double up = rnd_op(FE_UPWARD, P[2 * i + 1], b[2 * i], '-');
    P[2 * i] = lo;
    P[2 * i + 1] = up;
  }
  orc_pidblas_mul_point(1, n, nrhs, n, R, P, r, nthreads);
  if (E_in)
    memcpy(E, E_in, sizeof(double) * 2 * nn);
  else
    orc_pidblas_mul_point(1, n, n, n, R, A, E, nthreads);
  for (int i = 0; i < n; ++i) {
    const long o = i + (long)i * n;
    const double lo = rnd_op(FE_DOWNWARD, E[2 * o], 1.0, '-');
    const double up = rnd_op(FE_UPWARD, E[2 * o + 1], 1.0, '-');
    E[2 * o] = lo;
    E[2 * o + 1] = up;
  }
  const double G = norminf_sup(n, n, E);
  *bound = G;
  if (G >= 1.0) {
    free(buf);
    return 2;
  }
  const double t = norminf_sup(n, nrhs, r);
  const double d_lo = rnd_op(FE_DOWNWARD, 1.0, G, '-'), d_up = rnd_op(FE_UPWARD, 1.0, G, '-');
  const double q[4] = {rnd_op(FE_DOWNWARD, t, d_lo, '/'), rnd_op(FE_DOWNWARD, t, d_up, '/'),
                       rnd_op(FE_DOWNWARD, t, d_lo, '/'), rnd_op(FE_DOWNWARD, t, d_up, '/')};
  const double u4[4] = {rnd_op(FE_UPWARD, t, d_lo, '/'), rnd_op(FE_UPWARD, t, d_up, '/'),
                        rnd_op(FE_UPWARD, t, d_lo, '/'), rnd_op(FE_UPWARD, t, d_up, '/')};
  double g_lo = q[0], g_up = u4[0];
  for (int c = 1; c < 4; ++c) {
    if (q[c] < g_lo) g_lo = q[c];
    if (g_up < u4[c]) g_up = u4[c];
  }
  for (long i = 0; i < nn; ++i) {  /* E -> kv abs(E) */
    const double lo = E[2 * i], up = E[2 * i + 1];
    if (lo >= 0.0) continue;
    if (up <= 0.0) {
      E[2 * i] = -up;
      E[2 * i + 1] = -lo;
    } else {
      E[2 * i] = 0.0;
      E[2 * i + 1] = (-lo < up) ? up : -lo;
    }
  }
  for (long i = 0; i < nv; ++i) {
    T[2 * i] = g_lo;
    T[2 * i + 1] = g_up;
  }
  orc_pidblas_mulmm(n, nrhs, n, E, T, H, nthreads);
  for (long i = 0; i < nv; ++i) {
    const double u = rnd_op(FE_UPWARD, kv_abs_sup(r[2 * i], r[2 * i + 1]), H[2 * i + 1], '+');
    x[2 * i] = rnd_op(FE_DOWNWARD, -u, mx[i], '+');
    x[2 * i + 1] = rnd_op(FE_UPWARD, u, mx[i], '+');
  }
  free(buf);
  return 0;
}

/* ---------------------------------------------------------------------------
 * imats::eigsymge's verification (vcp/imats.hpp:419-522, Miyajima's
 * enclosure of the eigenvalues of A x = lambda B x) given the approximate
 * eigenvectors X and eigenvalues lambda of the midpoints and Y = inv(mid(B X)).
 * The reference's products are of two kinds: on its pidblas matrices the
 * pidblas hooks (midrad dgemm chains: [A] X, [B] X, Y [BX]); on its local
 * imats objects the base class's loops in kv interval arithmetic:
 *   R = Y C     imats::mul_m_im 'M' x 'M' (:203-213): c = 0; c += Y(i,j) * C(j,k)
 *               for j ascending, each product the kv product of [y, y] and C(j,k)
 *   |R| e       imats::mul_im_m 'M' x 'C' (:88-97): c = R(i,0); c = R(i,j) + c
 * C_in, BX_in, R_in, S_in (kv, n x n), when given, replace [A] X, [B] X,
 * Y C and Y [BX] (the tensor-core form's products).  lam (n kv) receives the
 * enclosures after the overlap merge (merge = 1) or before it; *bound the
 * sup of ||Y BX - I||.  Returns 0, or 2 when that bound is >= 1.
 * ------------------------------------------------------------------------- */
static void kv_mul_iv(double xl, double xu, double yl, double yu, double* lo, double* up) {
  const double a[4] = {rnd_op2(FE_DOWNWARD, xl, yl), rnd_op2(FE_DOWNWARD, xl, yu),
                       rnd_op2(FE_DOWNWARD, xu, yl), rnd_op2(FE_DOWNWARD, xu, yu)};
  const double b[4] = {rnd_op2(FE_UPWARD, xl, yl), rnd_op2(FE_UPWARD, xl, yu),
                       rnd_op2(FE_UPWARD, xu, yl), rnd_op2(FE_UPWARD, xu, yu)};
  double l = a[0], u = b[0];
  for (int c = 1; c < 4; ++c) {  /* std::min_element / max_element: first extreme */
    if (a[c] < l) l = a[c];
    if (u < b[c]) u = b[c];
  }
  *lo = l;
  *up = u;
}
static void kv_abs_inplace(long count, double* X) {
  for (long i = 0; i < count; ++i) {
    const double lo = X[2 * i], up = X[2 * i + 1];
    if (lo >= 0.0) continue;
    if (up <= 0.0) {
      X[2 * i] = -up;
      X[2 * i + 1] = -lo;
    } else {
      X[2 * i] = 0.0;
      X[2 * i + 1] = (-lo < up) ? up : -lo;
    }
  }
}
/* imats::mul_im_m 'M' x 'C' with the ones vector: interval row sums */
static void kv_row_sums(int n, const double* X, double* out) {
  for (int i = 0; i < n; ++i) {
    double lo = X[2 * i], up = X[2 * i + 1];
    for (int j = 1; j < n; ++j) {
      const long o = i + (long)j * n;
      lo = rnd_op(FE_DOWNWARD, X[2 * o], lo, '+');
      up = rnd_op(FE_UPWARD, X[2 * o + 1], up, '+');
    }
    out[2 * i] = lo;
    out[2 * i + 1] = up;
  }
}

void orc_imats_mul_m_im_naive(int m, int n, int k, const double* Y, const double* C, double* R) {
  /* R (m x n) = Y (m x k point) C (k x n kv), kv arithmetic, j ascending */
  for (long t = 0; t < 2L * m * n; ++t) R[t] = 0.0;
  for (int kk = 0; kk < n; ++kk)
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < m; ++i) {
        const double y = Y[i + (long)j * m];
        const long cj = j + (long)kk * k, o = i + (long)kk * m;
        double pl, pu;
        kv_mul_iv(y, y, C[2 * cj], C[2 * cj + 1], &pl, &pu);
        R[2 * o] = rnd_op(FE_DOWNWARD, R[2 * o], pl, '+');
        R[2 * o + 1] = rnd_op(FE_UPWARD, R[2 * o + 1], pu, '+');
      }
}

void orc_eig_merge(int n, double* lam) {
  for (int i = 0; i < n; ++i) {
    int j = 0;
    for (;;) {
      if (i != j) {
        double *x = lam + 2 * i, *y = lam + 2 * j;
        const int ov = x[0] <= y[1] && y[0] <= x[1];
        if (ov && (x[0] != y[0] || x[1] != y[1])) {
          x[0] = (y[0] < x[0]) ? y[0] : x[0];  /* std::min(x, y) = y < x ? y : x */
          x[1] = (x[1] < y[1]) ? y[1] : x[1];  /* std::max(x, y) = x < y ? y : x */
          y[0] = x[0];
          y[1] = x[1];
          j = 0;
          continue;
        }
      }
      if (++j == n) break;
    }
  }
}

int orc_ieigsymge(int n, const double* A, const double* B, const double* X, const double* lambda,
                  const double* Y, const double* C_in, const double* BX_in, const double* R_in,
                  const double* S_in, double* lam, double* bound, int merge, int nthreads) {
  const long nn = (long)n * n;
  double* buf = (double*)malloc(sizeof(double) * (8 * nn + 4 * n + n));
  if (!buf) return 1;
  double *C = buf, *BX = C + 2 * nn, *R = BX + 2 * nn, *S = R + 2 * nn, *Re = S + 2 * nn;
  double *Se = Re + 2 * n, *e = Se + 2 * n;
  for (int i = 0; i < n; ++i) e[i] = 1.0;
  if (C_in) memcpy(C, C_in, sizeof(double) * 2 * nn);
  else orc_pidblas_mul_point(0, n, n, n, A, X, C, nthreads);
  if (BX_in) memcpy(BX, BX_in, sizeof(double) * 2 * nn);
  else orc_pidblas_mul_point(0, n, n, n, B, X, BX, nthreads);
  for (int j = 0; j < n; ++j)  /* C(i,j) -= BX(i,j) * [lambda_j, lambda_j] */
    for (int i = 0; i < n; ++i) {
      const long o = i + (long)j * n;
      double pl, pu;
      kv_mul_iv(BX[2 * o], BX[2 * o + 1], lambda[j], lambda[j], &pl, &pu);
      const double lo = rnd_op(FE_DOWNWARD, C[2 * o], pu, '-');
      const double up = rnd_op(FE_UPWARD, C[2 * o + 1], pl, '-');
      C[2 * o] = lo;
      C[2 * o + 1] = up;
    }
  if (R_in) memcpy(R, R_in, sizeof(double) * 2 * nn);
  else orc_imats_mul_m_im_naive(n, n, n, Y, C, R);
  const double Rinf = norminf_sup(n, n, R);
  kv_abs_inplace(nn, R);
  kv_row_sums(n, R, Re);
  if (S_in) memcpy(S, S_in, sizeof(double) * 2 * nn);
  else orc_pidblas_mul_point(1, n, n, n, Y, BX, S, nthreads);
  for (int i = 0; i < n; ++i) {
    const long o = i + (long)i * n;
    const double lo = rnd_op(FE_DOWNWARD, S[2 * o], 1.0, '-');
    const double up = rnd_op(FE_UPWARD, S[2 * o + 1], 1.0, '-');
    S[2 * o] = lo;
    S[2 * o + 1] = up;
  }
  const double Sinf = norminf_sup(n, n, S);
  *bound = Sinf;
  if (Sinf >= 1.0) {
    free(buf);
    return 2;
  }
  kv_abs_inplace(nn, S);
  kv_row_sums(n, S, Se);
  const double d_lo = rnd_op(FE_DOWNWARD, 1.0, Sinf, '-'), d_up = rnd_op(FE_UPWARD, 1.0, Sinf, '-');
  const double q[4] = {rnd_op(FE_DOWNWARD, Rinf, d_lo, '/'), rnd_op(FE_DOWNWARD, Rinf, d_up, '/'),
                       rnd_op(FE_DOWNWARD, Rinf, d_lo, '/'), rnd_op(FE_DOWNWARD, Rinf, d_up, '/')};
  const double u4[4] = {rnd_op(FE_UPWARD, Rinf, d_lo, '/'), rnd_op(FE_UPWARD, Rinf, d_up, '/'),
                        rnd_op(FE_UPWARD, Rinf, d_lo, '/'), rnd_op(FE_UPWARD, Rinf, d_up, '/')};
  double g_lo = q[0], g_up = u4[0];
  for (int c = 1; c < 4; ++c) {
    if (q[c] < g_lo) g_lo = q[c];
    if (g_up < u4[c]) g_up = u4[c];
  }
  for (int i = 0; i < n; ++i) {
    double sl, su;
    kv_mul_iv(g_lo, g_up, Se[2 * i], Se[2 * i + 1], &sl, &su);  /* Se.mulsm(g): g * Se_i */
    const double u = rnd_op(FE_UPWARD, Re[2 * i + 1], su, '+');   /* Re.addmm(Se), sup */
    lam[2 * i] = rnd_op(FE_DOWNWARD, -u, lambda[i], '+');
    lam[2 * i + 1] = rnd_op(FE_UPWARD, u, lambda[i], '+');
  }
  if (merge) orc_eig_merge(n, lam);
  free(buf);
  return 0;
}

/* ---------------------------------------------------------------------------
 * vcp::ifma (vcp/ifma.hpp:48-139, the portable branch) and the product of
 * vcp::pidblas_fma::mulmm (vcp/pidblas_fma.hpp:46-80) built on it.
 * ------------------------------------------------------------------------- */
static double fma_dir(double a, double b, double c, int mode) {
  volatile double x = a, y = b, z = c;
  fesetround(mode);
  volatile double r = fma(x, y, z);
  fesetround(FE_TONEAREST);
  return r;
}

/* [rd, ru] = [ad, au] * [bd, bu] + [cd, cu]: the reference's sign cases. */
static void ifma_c(double au, double ad, double bu, double bd, double cu, double cd,
                   double* ru, double* rd) {
  double u = 0.0, d = 0.0, t;
  if (ad >= 0) {
    if (bd >= 0) {
      u = fma_dir(au, bu, cu, FE_UPWARD);
      d = fma_dir(ad, bd, cd, FE_DOWNWARD);
    } else if (bd <= 0 && bu >= 0) {
      u = fma_dir(au, bu, cu, FE_UPWARD);
      d = fma_dir(au, bd, cd, FE_DOWNWARD);
    } else if (bu <= 0) {
      u = fma_dir(ad, bu, cu, FE_UPWARD);
      d = fma_dir(au, bd, cd, FE_DOWNWARD);
    }
  } else if (ad <= 0 && au >= 0) {
    if (bd >= 0) {
      u = fma_dir(au, bu, cu, FE_UPWARD);
      d = fma_dir(ad, bu, cd, FE_DOWNWARD);
    } else if (bd <= 0 && bu >= 0) {
      t = fma_dir(au, bu, cu, FE_UPWARD);
      u = fma_dir(ad, bd, cu, FE_UPWARD);
      if (u < t) u = t;
      t = fma_dir(au, bd, cd, FE_DOWNWARD);
      d = fma_dir(ad, bu, cd, FE_DOWNWARD);
      if (d > t) d = t;
    } else if (bu <= 0) {
      u = fma_dir(ad, bd, cu, FE_UPWARD);
      d = fma_dir(au, bd, cd, FE_DOWNWARD);
    }
  } else if (au <= 0) {
    if (bd >= 0) {
      u = fma_dir(au, bd, cu, FE_UPWARD);
      d = fma_dir(ad, bu, cd, FE_DOWNWARD);
    } else if (bd <= 0 && bu >= 0) {
      u = fma_dir(ad, bd, cu, FE_UPWARD);
      d = fma_dir(ad, bu, cd, FE_DOWNWARD);
    } else if (bu <= 0) {
      u = fma_dir(ad, bd, cu, FE_UPWARD);
      d = fma_dir(au, bu, cd, FE_DOWNWARD);
    }
  }
  *ru = u;
  *rd = d;
}

void orc_ifma(long count, const double* A, const double* B, const double* C, double* R) {
  for (long i = 0; i < count; ++i) {
    double ru, rd;
    ifma_c(A[2 * i + 1], A[2 * i], B[2 * i + 1], B[2 * i], C[2 * i + 1], C[2 * i], &ru, &rd);
    R[2 * i] = rd;
    R[2 * i + 1] = ru;
  }
}

/* C (m x n) = fold of ifma over p = 0..k-1 from [0, 0] (the loop order of
 * pidblas_fma::mulmm: column of C, inner index, row). */
int orc_pidblas_fma_mulmm(int m, int n, int k, const double* A, const double* B, double* C,
                          int nthreads) {
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < m; ++i) {
      C[2 * ((long)i + (long)j * m)] = 0.0;
      C[2 * ((long)i + (long)j * m) + 1] = 0.0;
    }
    for (int p = 0; p < k; ++p) {
      for (int i = 0; i < m; ++i) {
        const double* a = A + 2 * ((long)i + (long)p * m);
        const double* b = B + 2 * ((long)p + (long)j * k);
        double* c = C + 2 * ((long)i + (long)j * m);
        double ru, rd;
        ifma_c(a[1], a[0], b[1], b[0], c[1], c[0], &ru, &rd);
        c[0] = rd;
        c[1] = ru;
      }
    }
  }
  (void)nthreads;
  return 0;
}

/* ---------------------------------------------------------------------------
 * Tensor-product basis matrices of the Legendre generator (the GPU's
 * vcpcu_tensor_basis_dev, restating phi_point_set, vcp/ldbase.hpp:355-374,
 * and the weight * uh^p factor of uhphiphi's element loop, :994-1001):
 *   out(i, q) = Ta(ia[i], qa) * Tb(ib[i], qb) [* s1(q)] [* s2(q)],
 *   q = qa * nqb + qb, each product the min of the four endpoint products
 *   rounded down and the max of the four rounded up; accumulate adds the
 *   entry already in out (rounded down / up).  Row by row: every rounding
 *   mode is set once per pass over a row's P entries.
 * ------------------------------------------------------------------------- */
static void imul_row(long P, const double* alo, const double* ahi, const double* b, long bstep,
                     double* lo, double* hi) {
  /* (alo, ahi)[q] times the kv pair b[q * bstep] for q < P */
  fesetround(FE_DOWNWARD);
  for (long q = 0; q < P; ++q) {
    volatile double a0 = alo[q], a1 = ahi[q], b0 = b[2 * q * bstep], b1 = b[2 * q * bstep + 1];
    volatile double p0 = a0 * b0, p1 = a0 * b1, p2 = a1 * b0, p3 = a1 * b1;
    lo[q] = fmin(fmin(p0, p1), fmin(p2, p3));
  }
  fesetround(FE_UPWARD);
  for (long q = 0; q < P; ++q) {
    volatile double a0 = alo[q], a1 = ahi[q], b0 = b[2 * q * bstep], b1 = b[2 * q * bstep + 1];
    volatile double p0 = a0 * b0, p1 = a0 * b1, p2 = a1 * b0, p3 = a1 * b1;
    hi[q] = fmax(fmax(p0, p1), fmax(p2, p3));
  }
  fesetround(FE_TONEAREST);
}

int orc_tensor_basis(int nb, const int* ia, const int* ib, int nt, const double* Ta,
                     const double* Tb, int nqa, int nqb, const double* s1, const double* s2,
                     double* out, long ld, int transposed, int accumulate, int nthreads) {
  const long P = (long)nqa * nqb;
  if (nb <= 0 || P <= 0) return 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    double* buf = malloc(sizeof(double) * 6 * P);
    double *alo = buf, *ahi = buf + P, *blo = buf + 2 * P, *bhi = buf + 3 * P;
    double* tb = buf + 4 * P; /* kv of Tb(ib[i], qb) expanded over q */
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
    for (int i = 0; i < nb; ++i) {
      const int a = ia[i], b = ib[i];
      double* o0 = transposed ? out + 2 * (long)i * ld : out + 2 * (long)i;
      const long ostep = transposed ? 1 : ld;
      if (a < 0 || a >= nt || b < 0 || b >= nt) {
        for (long q = 0; q < P; ++q) o0[2 * q * ostep] = o0[2 * q * ostep + 1] = NAN;
        continue;
      }
      for (long q = 0; q < P; ++q) {
        const long qa = q / nqb, qb = q - qa * nqb;
        alo[q] = Ta[2 * (a + qa * nt)];
        ahi[q] = Ta[2 * (a + qa * nt) + 1];
        tb[2 * q] = Tb[2 * (b + qb * nt)];
        tb[2 * q + 1] = Tb[2 * (b + qb * nt) + 1];
      }
      imul_row(P, alo, ahi, tb, 1, blo, bhi);
      double *clo = blo, *chi = bhi, *dlo = alo, *dhi = ahi;
      if (s1) {
        imul_row(P, clo, chi, s1, 1, dlo, dhi);
        double* t = clo; clo = dlo; dlo = t;
        t = chi; chi = dhi; dhi = t;
      }
      if (s2) {
        imul_row(P, clo, chi, s2, 1, dlo, dhi);
        double* t = clo; clo = dlo; dlo = t;
        t = chi; chi = dhi; dhi = t;
      }
      if (accumulate) {
        fesetround(FE_DOWNWARD);
        for (long q = 0; q < P; ++q) {
          volatile double x = clo[q], y = o0[2 * q * ostep];
          clo[q] = x + y;
        }
        fesetround(FE_UPWARD);
        for (long q = 0; q < P; ++q) {
          volatile double x = chi[q], y = o0[2 * q * ostep + 1];
          chi[q] = x + y;
        }
        fesetround(FE_TONEAREST);
      }
      for (long q = 0; q < P; ++q) {
        o0[2 * q * ostep] = clo[q];
        o0[2 * q * ostep + 1] = chi[q];
      }
    }
    free(buf);
  }
  (void)nthreads;
  return 0;
}

/* ---------------------------------------------------------------------------
 * pddblas (vcp/pddblas.hpp): the Ozaki-scheme dd product of the reference,
 * restated for the CPU baseline and for the accuracy comparison with the
 * GPU's dd product.  dd values are kv-layout pairs {a1, a2}; the dd addition
 * is the one of the project's kv stand-in (oracle/kvshim/kv/dd.hpp: TwoSum
 * of both words, Dekker renormalisations), in round-to-nearest.
 *   split geometry  pddblas_assist::ceil_log2 / split_shift / split_bits /
 *                   max_slices (:54-78)
 *   split_row/col   one sigma = 2^(e + s) per row / column, q = (a1 + sigma)
 *                   - sigma, the remainder T -= q in dd (:82-154)
 *   ozaki_acc       t = p + q ascending, p ascending, each slice product a
 *                   round-to-nearest dgemm (exact by construction), its
 *                   non-zero entries added into C in dd (:160-193)
 * ------------------------------------------------------------------------- */
static void dd_twosum(double a, double b, double* s, double* e) {
  volatile double vs = a + b;
  volatile double bb = vs - a;
  *s = vs;
  *e = (a - (vs - bb)) + (b - bb);
}
static void dd_fasttwosum(double a, double b, double* s, double* e) {
  volatile double vs = a + b;
  *s = vs;
  *e = b - (vs - a);
}
static void dd_add(double x1, double x2, double y1, double y2, double* r1, double* r2) {
  double s, e, t, f;
  dd_twosum(x1, y1, &s, &e);
  dd_twosum(x2, y2, &t, &f);
  e += t;
  dd_fasttwosum(s, e, &s, &e);
  e += f;
  dd_fasttwosum(s, e, r1, r2);
}

static int pdd_ceil_log2(int k) {
  int r = 0, t = 1;
  while (t < k) {
    t *= 2;
    ++r;
  }
  return r;
}
static int pdd_split_shift(int k) { return (51 + pdd_ceil_log2(k) + 1) / 2; }
static int pdd_split_bits(int k) {
  int b = 52 - pdd_split_shift(k);
  return b < 1 ? 1 : b;
}
static int pdd_max_slices(int k) { return 110 / pdd_split_bits(k) + 2; }

/* Split the dd array X (rows x cols, column-major, kv pairs) into slices
 * (rows x cols doubles each, appended to *D), one sigma per row (by_row) or
 * per column, with split parameter kk (the inner dimension).  Returns the
 * number of slices. */
static int pdd_split(const double* X, int rows, int cols, int by_row, int kk, double** D) {
  const int s = pdd_split_shift(kk), smax = pdd_max_slices(kk);
  const long cnt = (long)rows * cols;
  double* T = malloc(sizeof(double) * 2 * (cnt > 0 ? cnt : 1));
  memcpy(T, X, sizeof(double) * 2 * cnt);
  double* out = malloc(sizeof(double) * (size_t)smax * (cnt > 0 ? cnt : 1));
  int ns = 0;
  for (int p = 0; p < smax; ++p) {
    double* S = out + (size_t)p * cnt;
    memset(S, 0, sizeof(double) * cnt);
    int nonzero = 0;
    const int outer = by_row ? rows : cols, inner = by_row ? cols : rows;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : nonzero) if (cnt > 65536)
#endif
    for (int o = 0; o < outer; ++o) {
      fesetround(FE_TONEAREST);
      double mu = 0.0;
      for (int t = 0; t < inner; ++t) {
        const long idx = by_row ? o + (long)t * rows : t + (long)o * rows;
        const double a = fabs(T[2 * idx]);
        if (a > mu) mu = a;
      }
      if (mu == 0.0) continue;
      int e;
      frexp(mu, &e);
      const double sigma = ldexp(1.0, e + s);
      for (int t = 0; t < inner; ++t) {
        const long idx = by_row ? o + (long)t * rows : t + (long)o * rows;
        volatile double v = T[2 * idx] + sigma;
        volatile double q = v - sigma;
        if (q != 0.0) {
          S[idx] = q;
          double r1, r2;
          dd_add(T[2 * idx], T[2 * idx + 1], -q, -0.0, &r1, &r2);
          T[2 * idx] = r1;
          T[2 * idx + 1] = r2;
          nonzero = 1;
        }
      }
    }
    if (!nonzero) break;
    ++ns;
  }
  free(T);
  *D = out;
  return ns;
}

/* C (m x n dd) += sum of op(DA[p]) DB[q] over slice pairs, op(DA[p]) m x k
 * (stored k x m when transA). */
static void pdd_ozaki_acc(const double* DA, int na, long sa, int transA, const double* DB, int nb,
                          long sb, int m, int n, int k, double* C, int nthreads) {
  if (na == 0 || nb == 0) return;
  const int limit = pdd_max_slices(k);
  const long mn = (long)m * n;
  double* P = malloc(sizeof(double) * (mn > 0 ? mn : 1));
  double* At = transA ? malloc(sizeof(double) * ((long)m * k > 0 ? (long)m * k : 1)) : NULL;
  for (int t = 0; t < limit; ++t) {
    for (int p = 0; p <= t; ++p) {
      const int q = t - p;
      if (p >= na || q >= nb) continue;
      const double* Ap = DA + (size_t)p * sa;
      if (transA) { /* the k x m slice transposed to m x k */
        for (int i = 0; i < m; ++i)
          for (int l = 0; l < k; ++l) At[i + (long)l * m] = Ap[l + (long)i * k];
        Ap = At;
      }
      orc_rmatmul_ld(m, k, n, Ap, m, DB + (size_t)q * sb, k, P, m, 0, nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (mn > 65536) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
#endif
      for (long idx = 0; idx < mn; ++idx)
        if (P[idx] != 0.0) {
          double r1, r2;
          dd_add(C[2 * idx], C[2 * idx + 1], P[idx], 0.0, &r1, &r2);
          C[2 * idx] = r1;
          C[2 * idx + 1] = r2;
        }
    }
  }
  free(P);
  free(At);
}

/* pddblas::mulmm (vcp/pddblas.hpp:318-376), GEMM naming: C (m x n) = A (m x k)
 * B (k x n), dd kv pairs, column-major. */
static void dd_mul(double x1, double x2, double y1, double y2, double* r1, double* r2) {
  volatile double p = x1 * y1;
  double e = fma(x1, y1, -p);
  volatile double t2 = x2 * y1;
  volatile double t = fma(x1, y2, t2);
  e += t;
  dd_fasttwosum(p, e, r1, r2);
}

int orc_pddblas_mulmm(int m, int n, int k, const double* A, const double* B, double* C,
                      int nthreads) {
  for (long i = 0; i < 2L * m * n; ++i) C[i] = 0.0;
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  /* the scalar ('S', 1 x 1) shortcuts of pddblas::mulmm (:319-336) */
  if (m == 1 && k == 1 && n == 1) { /* c = a * b */
    dd_mul(A[0], A[1], B[0], B[1], C, C + 1);
    return 0;
  }
  if (m == 1 && k == 1) { /* c = B, c[i] *= a */
    for (long i = 0; i < (long)n; ++i) dd_mul(B[2 * i], B[2 * i + 1], A[0], A[1], C + 2 * i, C + 2 * i + 1);
    return 0;
  }
  if (k == 1 && n == 1) { /* c = A, c[i] *= b */
    for (long i = 0; i < (long)m; ++i) dd_mul(A[2 * i], A[2 * i + 1], B[0], B[1], C + 2 * i, C + 2 * i + 1);
    return 0;
  }
  double *DA, *DB;
  const int na = pdd_split(A, m, k, 1, k, &DA);
  const int nb = pdd_split(B, k, n, 0, k, &DB);
  pdd_ozaki_acc(DA, na, (long)m * k, 0, DB, nb, (long)k * n, m, n, k, C, nthreads);
  free(DA);
  free(DB);
  return 0;
}

/* pddblas::mulltmm (vcp/pddblas.hpp:379-409): C (nc x nc) = A^T A for A
 * (m x nc), the lower triangle then copied from the upper one. */
int orc_pddblas_mulltmm(int m, int nc, const double* A, double* C, int nthreads) {
  for (long i = 0; i < 2L * nc * nc; ++i) C[i] = 0.0;
  if (m <= 0 || nc <= 0) return 0;
  if (m == 1 && nc == 1) { /* 'S': a * a (:380-384) */
    dd_mul(A[0], A[1], A[0], A[1], C, C + 1);
    return 0;
  }
  double* DA;
  const int na = pdd_split(A, m, nc, 0, m, &DA);
  pdd_ozaki_acc(DA, na, (long)m * nc, 1, DA, na, (long)m * nc, nc, nc, m, C, nthreads);
  free(DA);
  for (int i = 0; i < nc; ++i)
    for (int j = i + 1; j < nc; ++j) {
      C[2 * (j + (long)nc * i)] = C[2 * (i + (long)nc * j)];
      C[2 * (j + (long)nc * i) + 1] = C[2 * (i + (long)nc * j) + 1];
    }
  return 0;
}

/* ---------------------------------------------------------------------------
 * Measured FP64 peak of the host cores (the denominator of the CPU port's
 * fraction of peak): every thread runs 16 independent fused multiply-add
 * chains (two lanes each on NEON) for about `seconds`; returns the aggregate
 * GFLOP/s (2 flops per lane per FMA).
 * ------------------------------------------------------------------------- */
#include <time.h>
static double orc_now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

double orc_fp64_peak(double seconds, int nthreads) {
  double total_flops = 0.0;
  const double t0 = orc_now();
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(+ : total_flops)
#endif
  {
    double flops = 0.0, sink = 0.0;
#if defined(__aarch64__)
    float64x2_t acc[16];
    for (int i = 0; i < 16; ++i) acc[i] = vdupq_n_f64(0.5 + i);
    const float64x2_t a = vdupq_n_f64(0.9999999), b = vdupq_n_f64(1e-9);
    do {
      for (int it = 0; it < (1 << 16); ++it)
        for (int i = 0; i < 16; ++i) acc[i] = vfmaq_f64(acc[i], a, b);
      flops += 16.0 * 2 * 2 * (1 << 16);
    } while (orc_now() - t0 < seconds);
    for (int i = 0; i < 16; ++i) sink += vgetq_lane_f64(acc[i], 0) + vgetq_lane_f64(acc[i], 1);
#else
    double acc[16];
    for (int i = 0; i < 16; ++i) acc[i] = 0.5 + i;
    do {
      for (int it = 0; it < (1 << 16); ++it)
        for (int i = 0; i < 16; ++i) acc[i] = fma(acc[i], 0.9999999, 1e-9);
      flops += 16.0 * 2 * (1 << 16);
    } while (orc_now() - t0 < seconds);
    for (int i = 0; i < 16; ++i) sink += acc[i];
#endif
    if (sink == 12345.678) flops += 1.0; /* keeps the chains live */
    total_flops += flops;
  }
  (void)nthreads;
  return total_flops / (orc_now() - t0) * 1e-9;
}
