// ref_wrap.cpp -- recipe that compiles the reference's own CPU path into
// oracle/_ref/libvcpref.so (see oracle/build.py).  TEST INFRASTRUCTURE ONLY.
//
// Included unmodified from the reference tree (-I<reference> -I<reference>/vblas):
//   vblas/rmatmul.hpp   -- the vblas directed-rounding GEMM (backend chosen by
//                          the compiler flags: AVX2+FMA on x86_64, NEON on Arm)
//   vcp/pidblas.hpp     -- the pidblas interval policy (with vcp/pdblas.hpp,
//                          vcp/imats.hpp, vcp/matrix.hpp)
// kv (interval, hwround) is absent and comes from oracle/kvshim.  pdblas calls
// the Fortran BLAS symbol dgemm_; this file provides dgemm_ (and ddot_,
// dgemv_, dsyrk_) on top of the reference rmatmul with the direction taken
// from the calling thread's current rounding mode, which is what pidblas sets
// through kv::hwround before each call (vcp/pidblas.hpp:264-281), and
// dgetrf_ / dgetri_ (a plain LU) for the inverse of imats::linearsolve.
#include <algorithm>
#include <cfenv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rmatmul.hpp"

#include <kv/interval.hpp>
#include <kv/hwround.hpp>
#include <vcp/pidblas.hpp>
#include <vcp/pidblas_fma.hpp>
#include <vcp/ifma.hpp>
#include <vcp/matrix.hpp>
#include <kv/dd.hpp>
#include <vcp/pddblas.hpp>
#include <vcp/vcp_portable_fio.hpp>

namespace {
int current_direction() {
  switch (std::fegetround()) {
    case FE_UPWARD: return 1;
    case FE_DOWNWARD: return -1;
    default: return 0;
  }
}
[[noreturn]] void unsupported(const char* what) {
  std::fprintf(stderr, "ref_wrap: unsupported BLAS call pattern: %s\n", what);
  std::abort();
}
}  // namespace

extern "C" {

// C = A * B for the pattern pdblas::mulmm uses (vcp/pdblas.hpp:91-110):
// trans "N","N", alpha 1, beta 0, lda = m, ldb = k, ldc = m.
// Also trans "T","N" with lda = k, the slice products of pddblas::mulltmm
// (vcp/pddblas.hpp:160-193): op(A) = A^T is transposed into a copy first.
void dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* alpha, const double* A, int* lda,
            const double* B, int* ldb, double* beta, double* C, int* ldc) {
  const bool tA = ta[0] == 'T';
  if ((ta[0] != 'N' && !tA) || tb[0] != 'N' || *alpha != 1.0 || *beta != 0.0 ||
      *lda != (tA ? *k : *m) || *ldb != *k || *ldc != *m)
    unsupported("dgemm_");
  if (!tA) {
    rmatmul(*m, *k, *n, A, B, C, current_direction());
    return;
  }
  std::vector<double> At((size_t)(*m) * (*k));
  for (int i = 0; i < *m; ++i)
    for (int p = 0; p < *k; ++p) At[i + (size_t)p * (*m)] = A[p + (size_t)i * (*lda)];
  rmatmul(*m, *k, *n, At.data(), B, C, current_direction());
}

// The double-precision solves of pddblas's refinements
// (vcp/pddblas.hpp:413-563).  LAPACK is absent here: project-written
// substitutions on the project-written LU above (dgetrs_, trans "N"), an
// upper Cholesky factor (dpotrf_, uplo "U", as pdblas::Cholesky calls it,
// vcp/pdblas.hpp:207-222) and the two triangular solves pddblas::Cholesky
// makes (dtrsm_ "L","U","T","N" and "R","U","N","N", alpha 1).  Any
// approximate solves serve the refinement: it converges to the same dd
// result within its accuracy.
void dgetrs_(char* trans, int* n, int* nrhs, double* A, int* lda, int* ipiv, double* B,
             int* ldb, int* info) {
  if (trans[0] != 'N') unsupported("dgetrs_");
  const int N = *n, ld = *lda;
  *info = 0;
  for (int c = 0; c < *nrhs; ++c) {
    double* e = B + (long)c * (*ldb);
    for (int j = 0; j < N; ++j) std::swap(e[j], e[ipiv[j] - 1]);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < i; ++j) e[i] -= A[i + (long)j * ld] * e[j];
    for (int i = N - 1; i >= 0; --i) {
      for (int j = i + 1; j < N; ++j) e[i] -= A[i + (long)j * ld] * e[j];
      e[i] /= A[i + (long)i * ld];
    }
  }
}

void dpotrf_(char* uplo, int* n, double* A, int* lda, int* info) {
  if (uplo[0] != 'U') unsupported("dpotrf_");
  const int N = *n, ld = *lda;
  *info = 0;
  for (int j = 0; j < N; ++j) {  // A = U^T U, U in the upper triangle
    double d = A[j + (long)j * ld];
    for (int p = 0; p < j; ++p) d -= A[p + (long)j * ld] * A[p + (long)j * ld];
    if (!(d > 0.0)) {
      *info = j + 1;
      return;
    }
    d = std::sqrt(d);
    A[j + (long)j * ld] = d;
    for (int c = j + 1; c < N; ++c) {
      double t = A[j + (long)c * ld];
      for (int p = 0; p < j; ++p) t -= A[p + (long)j * ld] * A[p + (long)c * ld];
      A[j + (long)c * ld] = t / d;
    }
  }
}

void dtrsm_(char* side, char* uplo, char* transa, char* diag, int* m, int* n, double* alpha,
            double* A, int* lda, double* B, int* ldb) {
  const int M = *m, N = *n, la = *lda, lb = *ldb;
  if (uplo[0] != 'U' || diag[0] != 'N' || *alpha != 1.0) unsupported("dtrsm_");
  if (side[0] == 'L' && transa[0] == 'T') {  // U^T X = B, column by column
    for (int c = 0; c < N; ++c)
      for (int i = 0; i < M; ++i) {
        double t = B[i + (long)c * lb];
        for (int p = 0; p < i; ++p) t -= A[p + (long)i * la] * B[p + (long)c * lb];
        B[i + (long)c * lb] = t / A[i + (long)i * la];
      }
  } else if (side[0] == 'R' && transa[0] == 'N') {  // X U = B, row by row
    for (int r = 0; r < M; ++r)
      for (int j = 0; j < N; ++j) {
        double t = B[r + (long)j * lb];
        for (int p = 0; p < j; ++p) t -= B[r + (long)p * lb] * A[p + (long)j * la];
        B[r + (long)j * lb] = t / A[j + (long)j * la];
      }
  } else {
    unsupported("dtrsm_");
  }
}

double ddot_(int* n, const double* x, int* incx, const double* y, int* incy) {
  if (*incx != 1 || *incy != 1) unsupported("ddot_");
  double c = 0.0;
  rmatmul(1, *n, 1, x, y, &c, current_direction());
  return c;
}

void dgemv_(char* t, int* m, int* n, double* alpha, const double* A, int* lda, const double* x,
            int* incx, double* beta, double* y, int* incy) {
  if (t[0] != 'N' || *alpha != 1.0 || *beta != 0.0 || *lda != *m || *incx != 1 || *incy != 1)
    unsupported("dgemv_");
  rmatmul(*m, *n, 1, A, x, y, current_direction());
}

// Upper triangle of A^T A (vcp/pdblas.hpp:138-146: uplo "U", trans "T").
void dsyrk_(char* uplo, char* trans, int* n, int* k, double* alpha, const double* A, int* lda,
            double* beta, double* C, int* ldc) {
  if (uplo[0] != 'U' || trans[0] != 'T' || *alpha != 1.0 || *beta != 0.0 || *lda != *k)
    unsupported("dsyrk_");
  std::vector<double> At((size_t)(*k) * (*n));
  for (int j = 0; j < *n; ++j)
    for (int p = 0; p < *k; ++p) At[j + (size_t)p * (*n)] = A[p + (size_t)j * (*lda)];
  std::vector<double> full((size_t)(*n) * (*n));
  rmatmul(*n, *k, *n, At.data(), A, full.data(), current_direction());
  for (int j = 0; j < *n; ++j)
    for (int i = 0; i <= j; ++i) C[i + (size_t)j * (*ldc)] = full[i + (size_t)j * (*n)];
}

// The approximate inverse R = inv(mid A) of imats::linearsolve
// (vcp/imats.hpp:299-300) comes from pdblas::inv (vcp/pdblas.hpp:180-205):
// dgetrf_ then dgetri_.  LAPACK is absent here; these two are a
// project-written LU with partial pivoting (first largest pivot) and the
// inverse by forward / back substitution of the unit columns, under the
// caller's rounding mode.  Any approximate inverse serves the verification;
// the same R is handed to the GPU path, so results are compared on equal R.
void dgetrf_(int* m, int* n, double* A, int* lda, int* ipiv, int* info) {
  const int M = *m, N = *n, ld = *lda;
  *info = 0;
  for (int j = 0; j < (M < N ? M : N); ++j) {
    int p = j;
    for (int i = j + 1; i < M; ++i)
      if (std::fabs(A[i + (long)j * ld]) > std::fabs(A[p + (long)j * ld])) p = i;
    ipiv[j] = p + 1;
    if (A[p + (long)j * ld] == 0.0) {
      if (*info == 0) *info = j + 1;
      continue;
    }
    if (p != j)
      for (int c = 0; c < N; ++c) std::swap(A[j + (long)c * ld], A[p + (long)c * ld]);
    for (int i = j + 1; i < M; ++i) A[i + (long)j * ld] /= A[j + (long)j * ld];
    for (int c = j + 1; c < N; ++c)
      for (int i = j + 1; i < M; ++i) A[i + (long)c * ld] -= A[i + (long)j * ld] * A[j + (long)c * ld];
  }
}

void dgetri_(int* n, double* A, int* lda, int* ipiv, double* work, int* lwork, int* info) {
  const int N = *n, ld = *lda;
  *info = 0;
  if (*lwork == -1) {  // workspace query
    work[0] = N > 0 ? N : 1;
    return;
  }
  std::vector<double> X((size_t)N * N, 0.0), e(N);
  for (int c = 0; c < N; ++c) {
    for (int i = 0; i < N; ++i) e[i] = i == c ? 1.0 : 0.0;
    for (int j = 0; j < N; ++j) std::swap(e[j], e[ipiv[j] - 1]);  // P e
    for (int i = 0; i < N; ++i)                                   // L y = P e
      for (int j = 0; j < i; ++j) e[i] -= A[i + (long)j * ld] * e[j];
    for (int i = N - 1; i >= 0; --i) {                            // U x = y
      for (int j = i + 1; j < N; ++j) e[i] -= A[i + (long)j * ld] * e[j];
      e[i] /= A[i + (long)i * ld];
    }
    for (int i = 0; i < N; ++i) X[i + (size_t)c * N] = e[i];
  }
  for (int c = 0; c < N; ++c)
    for (int i = 0; i < N; ++i) A[i + (long)c * ld] = X[i + (size_t)c * N];
}

// The approximate eigenpairs of imats::eigsymge (vcp/imats.hpp:427-434) come
// from pdblas::eigsymge (vcp/pdblas.hpp:334-375): dsygv_ with itype 1, jobz
// "V", uplo "U".  Project-written: Cholesky B = U^T U (upper triangle),
// cyclic Jacobi on U^-T A U^-1 to convergence, eigenvalues ascending in W,
// B-orthonormal eigenvectors X = U^-1 V in A, U in B.  Any approximate
// eigenpairs serve the verification; the same X is handed to the GPU path.
void dsygv_(int* itype, char* jobz, char* uplo, int* n, double* A, int* lda, double* B, int* ldb,
            double* W, double* work, int* lwork, int* info) {
  const int N = *n, la = *lda, lb = *ldb;
  *info = 0;
  if (*lwork == -1) {
    work[0] = 3.0 * (N > 0 ? N : 1);
    return;
  }
  if (*itype != 1 || jobz[0] != 'V' || uplo[0] != 'U') unsupported("dsygv_");
  std::vector<double> U((size_t)N * N, 0.0), M((size_t)N * N), V((size_t)N * N, 0.0);
  auto u = [&](int i, int j) -> double& { return U[i + (size_t)j * N]; };
  auto m = [&](int i, int j) -> double& { return M[i + (size_t)j * N]; };
  auto v = [&](int i, int j) -> double& { return V[i + (size_t)j * N]; };
  for (int j = 0; j < N; ++j) {  // B = U^T U
    for (int i = 0; i <= j; ++i) {
      double t = B[i + (long)j * lb];
      for (int k = 0; k < i; ++k) t -= u(k, i) * u(k, j);
      if (i == j) {
        if (!(t > 0.0)) {
          *info = N + j + 1;
          return;
        }
        u(j, j) = std::sqrt(t);
      } else {
        u(i, j) = t / u(i, i);
      }
    }
  }
  // M = U^-T A U^-1 (A symmetric from its upper triangle)
  std::vector<double> T((size_t)N * N);
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i)
      T[i + (size_t)j * N] = i <= j ? A[i + (long)j * la] : A[j + (long)i * la];
  for (int j = 0; j < N; ++j)  // T <- U^-T T (forward substitution, column j)
    for (int i = 0; i < N; ++i) {
      double t = T[i + (size_t)j * N];
      for (int k = 0; k < i; ++k) t -= u(k, i) * T[k + (size_t)j * N];
      T[i + (size_t)j * N] = t / u(i, i);
    }
  for (int i = 0; i < N; ++i)  // M <- T U^-1 (row i)
    for (int j = 0; j < N; ++j) {
      double t = T[i + (size_t)j * N];
      for (int k = 0; k < j; ++k) t -= m(i, k) * u(k, j);
      m(i, j) = t / u(j, j);
    }
  for (int i = 0; i < N; ++i) v(i, i) = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {  // cyclic Jacobi
    double off = 0.0;
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < j; ++i) off += m(i, j) * m(i, j);
    if (off == 0.0) break;
    for (int p = 0; p < N; ++p)
      for (int q = p + 1; q < N; ++q) {
        if (m(p, q) == 0.0) continue;
        const double th = (m(q, q) - m(p, p)) / (2.0 * m(p, q));
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s_ = t * c;
        for (int k = 0; k < N; ++k) {  // columns p, q
          const double a = m(k, p), b = m(k, q);
          m(k, p) = c * a - s_ * b;
          m(k, q) = s_ * a + c * b;
        }
        for (int k = 0; k < N; ++k) {  // rows p, q
          const double a = m(p, k), b = m(q, k);
          m(p, k) = c * a - s_ * b;
          m(q, k) = s_ * a + c * b;
        }
        for (int k = 0; k < N; ++k) {
          const double a = v(k, p), b = v(k, q);
          v(k, p) = c * a - s_ * b;
          v(k, q) = s_ * a + c * b;
        }
      }
  }
  std::vector<int> ord(N);
  for (int i = 0; i < N; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return m(a, a) < m(b, b); });
  for (int c = 0; c < N; ++c) {  // X(:, c) = U^-1 V(:, ord[c]) (back substitution)
    W[c] = m(ord[c], ord[c]);
    for (int i = N - 1; i >= 0; --i) {
      double t = v(i, ord[c]);
      for (int k = i + 1; k < N; ++k) t -= u(i, k) * A[k + (long)c * la];
      A[i + (long)c * la] = t / u(i, i);
    }
  }
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) B[i + (long)j * lb] = i <= j ? u(i, j) : 0.0;
}

// The remaining LAPACK / BLAS routines are referenced by pdblas's solver
// members (vcp/pdblas.hpp:159-376), which are off the GEMM path: they abort.
void dsymm_(char*, char*, int*, int*, double*, const double*, int*, const double*, int*, double*,
            double*, int*) { unsupported("dsymm_"); }
// pdblas::eigsym's dsyev_ (jobz "V", uplo "U", vcp/pdblas.hpp:259-289): the
// project-written dsygv_ above with B = I (eigenvalues ascending, orthonormal
// eigenvectors in A); pddblas::eigsym refines its result.
void dsyev_(char* jobz, char* uplo, int* n, double* A, int* lda, double* W, double* work,
            int* lwork, int* info) {
  const int N = *n;
  *info = 0;
  if (*lwork == -1) {
    work[0] = 3.0 * (N > 0 ? N : 1);
    return;
  }
  if (jobz[0] != 'V' || uplo[0] != 'U') unsupported("dsyev_");
  std::vector<double> I((size_t)N * N, 0.0);
  for (int i = 0; i < N; ++i) I[i + (size_t)i * N] = 1.0;
  int itype = 1, ldi = N;
  dsygv_(&itype, jobz, uplo, n, A, lda, I.data(), &ldi, W, work, lwork, info);
}
void dgesv_(int*, int*, double*, int*, int*, double*, int*, int*) { unsupported("dgesv_"); }

// The reference vblas entry point, unchanged.
void ref_rmatmul(int m, int n, int k, const double* A, const double* B, double* C, int rnd) {
  rmatmul(m, n, k, A, B, C, rnd);
}

// C = A * B through vcp::matrix<kv::interval<double>, vcp::pidblas>
// (operator* -> pidblas::mulmm, vcp/matrix.hpp:245-266).  GEMM naming:
// A m x k, B k x n, all in kv layout.
int ref_pidblas_mulmm(int m, int n, int k, const double* A, const double* B, double* C) {
  try {
    typedef kv::interval<double> I;
    vcp::matrix<I, vcp::pidblas> a, b, c;
    a.zeros(m, k);
    b.zeros(k, n);
    for (long i = 0; i < (long)m * k; ++i) a.data()[i] = I(A[2 * i], A[2 * i + 1]);
    for (long i = 0; i < (long)k * n; ++i) b.data()[i] = I(B[2 * i], B[2 * i + 1]);
    c = a * b;
    for (long i = 0; i < (long)m * n; ++i) {
      C[2 * i] = c.data()[i].lower();
      C[2 * i + 1] = c.data()[i].upper();
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

}  // extern "C"

namespace {
// Exposes pidblas's protected interval x point hooks (vcp/pidblas.hpp:90-236).
struct pidblas_open : vcp::pidblas {
  using vcp::pidblas::mul_im_m;
  using vcp::pidblas::mul_m_im;
  using vcp::pidblas::vmulmm;
  using vcp::pidblas::imid;
};
struct imats_open : vcp::imats<double, vcp::pdblas> {
  using vcp::imats<double, vcp::pdblas>::imid;
};
typedef kv::interval<double> I;
void fill_iv(vcp::mats<I>& X, int r, int c, const double* kvp) {
  X.zeros(r, c);
  for (long t = 0; t < (long)r * c; ++t) X.v[t] = I(kvp[2 * t], kvp[2 * t + 1]);
}
void fill_pt(vcp::pdblas& X, int r, int c, const double* p) {
  X.zeros(r, c);
  for (long t = 0; t < (long)r * c; ++t) X.v[t] = p[t];
}
void out_iv(const vcp::mats<I>& X, double* kvp) {
  for (long t = 0; t < (long)X.n; ++t) {
    kvp[2 * t] = X.v[t].lower();
    kvp[2 * t + 1] = X.v[t].upper();
  }
}
}  // namespace

extern "C" {

// pidblas::mul_im_m (side 0: [L] R) / mul_m_im (side 1: L [R]), GEMM naming.
int ref_pidblas_mul_point(int side, int m, int n, int k, const double* L, const double* R,
                          double* C) {
  try {
    pidblas_open iv;
    vcp::pdblas pt;
    vcp::imats<double, vcp::pdblas> c;
    if (side == 0) {
      fill_iv(iv, m, k, L);
      fill_pt(pt, k, n, R);
      iv.mul_im_m(pt, c);
    } else {
      fill_iv(iv, k, n, R);
      fill_pt(pt, m, k, L);
      iv.mul_m_im(pt, c);
    }
    out_iv(c, C);
    return 0;
  } catch (...) {
    return 1;
  }
}

// pidblas::mulltmm: C (n x n) = [A]^T [A], A k x n.
int ref_pidblas_mulltmm(int n, int k, const double* A, double* C) {
  try {
    pidblas_open a;
    fill_iv(a, k, n, A);
    vcp::mats<I> c;
    a.mulltmm(c);
    out_iv(c, C);
    return 0;
  } catch (...) {
    return 1;
  }
}

// pidblas::vmulmm: [A^T A] of a point A (k x n).
int ref_pidblas_vmulmm(int n, int k, const double* A, double* C) {
  try {
    vcp::pdblas a;
    fill_pt(a, k, n, A);
    pidblas_open c;
    c.vmulmm(a);
    out_iv(c, C);
    return 0;
  } catch (...) {
    return 1;
  }
}

// The bound of imats::linearsolve (vcp/imats.hpp:316-336): b = R [A] by
// pidblas::mul_m_im, b(i,i) -= 1, mats::norminf, upper end.
int ref_norm_I_minus_RA(int n, const double* R, const double* A, double* bound) {
  try {
    pidblas_open a;
    fill_iv(a, n, n, A);
    vcp::pdblas r;
    fill_pt(r, n, n, R);
    vcp::imats<double, vcp::pdblas> b;
    a.mul_m_im(r, b);
    for (int i = 0; i < n; ++i) b.v[i + n * i] -= 1.0;
    vcp::mats<I> g;
    b.norminf(g);
    *bound = g.v[0].upper();
    return 0;
  } catch (...) {
    return 1;
  }
}

// imats<double, pidblas>::linearsolve (vcp/imats.hpp:293-364), run as is: x
// (n x nrhs, kv layout).  R and mx receive the approximate inverse and
// solution it works with, formed the same way (imid, pdblas::inv,
// pdblas::mulmm; :299-302).  Returns 0, 2 when the reference throws
// vcp::verification_error (||RA - I|| >= 1), 1 on any other exception.
int ref_imats_linearsolve(int n, int nrhs, const double* A, const double* b, double* x,
                          double* R, double* mx) {
  try {
    pidblas_open a;
    fill_iv(a, n, n, A);
    imats_open bb;
    fill_iv(bb, n, nrhs, b);
    vcp::pdblas Rm, mb, mxm;
    a.imid(Rm);
    bb.imid(mb);
    Rm.inv();
    Rm.mulmm(mb, mxm);
    for (long t = 0; t < (long)n * n; ++t) R[t] = Rm.v[t];
    for (long t = 0; t < (long)n * nrhs; ++t) mx[t] = mxm.v[t];
    vcp::imats<double, vcp::pdblas> xx;
    a.linearsolve(bb, xx);
    out_iv(xx, x);
    return 0;
  } catch (vcp::verification_error&) {
    return 2;
  } catch (...) {
    return 1;
  }
}

}  // extern "C"

// imats<double, pidblas>::eigsymge (vcp/imats.hpp:419-522), run as is on A, B
// (n x n kv): lam receives the n eigenvalue enclosures (the diagonal it
// leaves), X, lambda and Y the approximate eigenvectors, eigenvalues and
// inverse of mid(B X) it works with, formed the same way (imid,
// pdblas::eigsymge, diag, pidblas::mul_im_m, imid, pdblas::inv).  Returns
// 0, 2 when the reference throws vcp::verification_error, 1 otherwise.
extern "C" int ref_imats_eigsymge(int n, const double* A, const double* B, double* lam,
                                  double* X, double* lambda, double* Y) {
  try {
    pidblas_open a, b;
    fill_iv(a, n, n, A);
    fill_iv(b, n, n, B);
    {
      vcp::pdblas mA, mB, Xm, app, Ym;
      a.imid(mA);
      b.imid(mB);
      mA.eigsymge(mB, Xm);
      mA.diag(app);
      pidblas_open bx;
      b.mul_im_m(Xm, bx);
      bx.imid(Ym);
      Ym.inv();
      for (long t = 0; t < (long)n * n; ++t) {
        X[t] = Xm.v[t];
        Y[t] = Ym.v[t];
      }
      for (int i = 0; i < n; ++i) lambda[i] = app.v[i];
    }
    a.eigsymge(b);
    for (int i = 0; i < n; ++i) {
      lam[2 * i] = a.v[i + (long)n * i].lower();
      lam[2 * i + 1] = a.v[i + (long)n * i].upper();
    }
    return 0;
  } catch (vcp::verification_error&) {
    return 2;
  } catch (...) {
    return 1;
  }
}

// vcp::save_portable / load_portable (vcp/vcp_portable_fio.hpp) of a
// vcp::matrix of each element type, the data in flat element layouts
// (type 1 int32, 2 double, 3 {lower, upper}, 4 {a1, a2}, 5 {lo.a1, lo.a2,
// up.a1, up.a2}).  Returns 0, 3 on vcp::io_error, 1 on anything else; a load
// also reports the file's rows and columns (and fills data when it is not
// null and large enough).
namespace {
typedef kv::interval<kv::dd> IDD;
void put_el(int& x, const void* d, long t) { x = ((const int*)d)[t]; }
void put_el(double& x, const void* d, long t) { x = ((const double*)d)[t]; }
void put_el(I& x, const void* d, long t) {
  const double* p = (const double*)d + 2 * t;
  x.assign(p[0], p[1]);
}
void put_el(kv::dd& x, const void* d, long t) {
  const double* p = (const double*)d + 2 * t;
  x.a1 = p[0];
  x.a2 = p[1];
}
void put_el(IDD& x, const void* d, long t) {
  const double* p = (const double*)d + 4 * t;
  x.lower().a1 = p[0];
  x.lower().a2 = p[1];
  x.upper().a1 = p[2];
  x.upper().a2 = p[3];
}
void get_el(const int& x, void* d, long t) { ((int*)d)[t] = x; }
void get_el(const double& x, void* d, long t) { ((double*)d)[t] = x; }
void get_el(const I& x, void* d, long t) {
  ((double*)d)[2 * t] = x.lower();
  ((double*)d)[2 * t + 1] = x.upper();
}
void get_el(const kv::dd& x, void* d, long t) {
  ((double*)d)[2 * t] = x.a1;
  ((double*)d)[2 * t + 1] = x.a2;
}
void get_el(const IDD& x, void* d, long t) {
  double* p = (double*)d + 4 * t;
  p[0] = x.lower().a1;
  p[1] = x.lower().a2;
  p[2] = x.upper().a1;
  p[3] = x.upper().a2;
}
template <class T> int vcpmat_save_t(const char* name, int rows, int cols, const void* data) {
  vcp::matrix<T> A;
  A.zeros(rows, cols);
  for (int j = 0; j < cols; ++j)
    for (int i = 0; i < rows; ++i) put_el(A(i, j), data, i + (long)j * rows);
  vcp::save_portable(A, name);
  return 0;
}
template <class T> int vcpmat_load_t(const char* name, int* rows, int* cols, void* data,
                                     long capacity) {
  vcp::matrix<T> A;
  vcp::load_portable(A, name);
  *rows = A.rowsize();
  *cols = A.columnsize();
  if (data && (long)A.rowsize() * A.columnsize() <= capacity)
    for (int j = 0; j < A.columnsize(); ++j)
      for (int i = 0; i < A.rowsize(); ++i) {
        const vcp::matrix<T>& cA = A;
        get_el(cA(i, j), data, i + (long)j * A.rowsize());
      }
  return 0;
}
}  // namespace

extern "C" {

int ref_vcpmat_save(const char* name, int type, int rows, int cols, const void* data) {
  try {
    switch (type) {
      case 1: return vcpmat_save_t<int>(name, rows, cols, data);
      case 2: return vcpmat_save_t<double>(name, rows, cols, data);
      case 3: return vcpmat_save_t<I>(name, rows, cols, data);
      case 4: return vcpmat_save_t<kv::dd>(name, rows, cols, data);
      case 5: return vcpmat_save_t<IDD>(name, rows, cols, data);
      default: return 1;
    }
  } catch (vcp::io_error&) {
    return 3;
  } catch (...) {
    return 1;
  }
}

int ref_vcpmat_load(const char* name, int type, int* rows, int* cols, void* data,
                    long capacity) {
  try {
    switch (type) {
      case 1: return vcpmat_load_t<int>(name, rows, cols, data, capacity);
      case 2: return vcpmat_load_t<double>(name, rows, cols, data, capacity);
      case 3: return vcpmat_load_t<I>(name, rows, cols, data, capacity);
      case 4: return vcpmat_load_t<kv::dd>(name, rows, cols, data, capacity);
      case 5: return vcpmat_load_t<IDD>(name, rows, cols, data, capacity);
      default: return 1;
    }
  } catch (vcp::io_error&) {
    return 3;
  } catch (...) {
    return 1;
  }
}

}  // extern "C"

extern "C" {

// vcp::ifma (vcp/ifma.hpp, the portable branch: VCP_USE_AVX512 undefined),
// elementwise over kv pairs.
void ref_ifma(long count, const double* A, const double* B, const double* C, double* R) {
  for (long i = 0; i < count; ++i) {
    double ru, rd;
    vcp::ifma(A[2 * i + 1], A[2 * i], B[2 * i + 1], B[2 * i], C[2 * i + 1], C[2 * i], ru, rd);
    R[2 * i] = rd;
    R[2 * i + 1] = ru;
  }
}

// C = A * B through vcp::matrix<kv::interval<double>, vcp::pidblas_fma>
// (pidblas_fma::mulmm, vcp/pidblas_fma.hpp:46-80).  GEMM naming, kv layout.
int ref_pidblas_fma_mulmm(int m, int n, int k, const double* A, const double* B, double* C) {
  try {
    vcp::matrix<I, vcp::pidblas_fma> a, b, c;
    a.zeros(m, k);
    b.zeros(k, n);
    for (long i = 0; i < (long)m * k; ++i) a.data()[i] = I(A[2 * i], A[2 * i + 1]);
    for (long i = 0; i < (long)k * n; ++i) b.data()[i] = I(B[2 * i], B[2 * i + 1]);
    c = a * b;
    for (long i = 0; i < (long)m * n; ++i) {
      C[2 * i] = c.data()[i].lower();
      C[2 * i + 1] = c.data()[i].upper();
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

}  // extern "C"

extern "C" {

// The pair as given (no renormalisation), as the restatement reads it.
static void set_dd(kv::dd& x, const double* p) {
  x.a1 = p[0];
  x.a2 = p[1];
}

// C = A * B through vcp::matrix<kv::dd, vcp::pddblas> (pddblas::mulmm,
// vcp/pddblas.hpp:318-376: Ozaki slices, RN dgemm, dd accumulation).
// GEMM naming, kv::dd pairs, column-major.
int ref_pddblas_mulmm(int m, int n, int k, const double* A, const double* B, double* C) {
  try {
    vcp::matrix<kv::dd, vcp::pddblas> a, b, c;
    a.zeros(m, k);
    b.zeros(k, n);
    for (long i = 0; i < (long)m * k; ++i) set_dd(a.data()[i], A + 2 * i);
    for (long i = 0; i < (long)k * n; ++i) set_dd(b.data()[i], B + 2 * i);
    c = a * b;
    for (long i = 0; i < (long)m * n; ++i) {
      C[2 * i] = c.data()[i].a1;
      C[2 * i + 1] = c.data()[i].a2;
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

// C = A^T A through pddblas::mulltmm (vcp/pddblas.hpp:379-409); A is m x nc.
int ref_pddblas_mulltmm(int m, int nc, const double* A, double* C) {
  try {
    vcp::matrix<kv::dd, vcp::pddblas> a, c;
    a.zeros(m, nc);
    for (long i = 0; i < (long)m * nc; ++i) set_dd(a.data()[i], A + 2 * i);
    c = ltransmul(a);
    for (long i = 0; i < (long)nc * nc; ++i) {
      C[2 * i] = c.data()[i].a1;
      C[2 * i + 1] = c.data()[i].a2;
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

}  // extern "C"

extern "C" {

// x = A \ b through vcp::matrix<kv::dd, vcp::pddblas> (pddblas::linearsolve,
// vcp/pddblas.hpp:413-474): LU in double, dd residuals by the Ozaki scheme.
int ref_pddblas_linearsolve(int n, int nrhs, const double* A, const double* b, double* x) {
  try {
    vcp::matrix<kv::dd, vcp::pddblas> a, bb, xx;
    a.zeros(n, n);
    bb.zeros(n, nrhs);
    for (long i = 0; i < (long)n * n; ++i) set_dd(a.data()[i], A + 2 * i);
    for (long i = 0; i < (long)n * nrhs; ++i) set_dd(bb.data()[i], b + 2 * i);
    xx = lss(a, bb);
    for (long i = 0; i < (long)n * nrhs; ++i) {
      x[2 * i] = xx.data()[i].a1;
      x[2 * i + 1] = xx.data()[i].a2;
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

// inv(A) (pddblas::inv, :477-486) and the upper Cholesky factor
// (pddblas::Cholesky, :490-563): which = 0 / 1.
int ref_pddblas_unary(int which, int n, const double* A, double* R) {
  try {
    vcp::matrix<kv::dd, vcp::pddblas> a, r;
    a.zeros(n, n);
    for (long i = 0; i < (long)n * n; ++i) set_dd(a.data()[i], A + 2 * i);
    if (which == 0)
      r = inv(a);
    else
      r = Cholesky(a);
    for (long i = 0; i < (long)n * n; ++i) {
      R[2 * i] = r.data()[i].a1;
      R[2 * i + 1] = r.data()[i].a2;
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

}  // extern "C"

extern "C" {

// pddblas::eigsym (vcp/pddblas.hpp:566-614) and eigsymge (:616-657) with
// eigenvectors, itep as given: the eigenvalues lam (n dd pairs) and the
// eigenvectors X (n x n dd pairs, columns).  B == NULL: the standard problem.
int ref_pddblas_eig(int n, const double* A, const double* B, int itep, double* lam, double* X) {
  try {
    vcp::matrix<kv::dd, vcp::pddblas> a, b, e, v;
    a.zeros(n, n);
    for (long i = 0; i < (long)n * n; ++i) set_dd(a.data()[i], A + 2 * i);
    if (B) {
      b.zeros(n, n);
      for (long i = 0; i < (long)n * n; ++i) set_dd(b.data()[i], B + 2 * i);
      eigsymge(a, b, e, v, itep);
    } else {
      eigsym(a, e, v, itep);
    }
    for (int i = 0; i < n; ++i) {
      lam[2 * i] = e.data()[i + (long)i * n].a1;
      lam[2 * i + 1] = e.data()[i + (long)i * n].a2;
    }
    for (long i = 0; i < (long)n * n; ++i) {
      X[2 * i] = v.data()[i].a1;
      X[2 * i + 1] = v.data()[i].a2;
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

}  // extern "C"
