// vcp_cuda/pddcuda.hpp -- vcp::pddcuda, the GPU drop-in for vcp::pddblas.
//
// Use exactly like pddblas (vcp/pddblas.hpp:204):
//     vcp::matrix< kv::dd, vcp::pddcuda > A, B, C;
//     C = A * B;            // pddcuda::mulmm   (pddblas::mulmm,   pddblas.hpp:318)
//     C = ltransmul(A);     // pddcuda::mulltmm (pddblas::mulltmm, pddblas.hpp:379)
//     x = lss(A, b);        // pddcuda::linearsolve (pddblas.hpp:413-474)
//     R = inv(A);           // pddcuda::inv         (:477-486)
//     U = Cholesky(A);      // pddcuda::Cholesky    (:490-563)
//     eigsym(A, E, V);      // pddcuda::eigsym / eigsymge (Ogita-Aishima, :221-314)
// The products are replaced by vcpcu_ddgemm (include/vcpcuda.h): the dd
// operands are scaled per row / column to w-bit integers, multiplied
// exactly on the tensor cores through residues modulo small primes, and
// rounded to the dd result -- the same product pddblas forms from
// error-free double slices (ozaki_acc), at least as accurate.  The
// refinement loops keep pddblas's steps, double-precision LAPACK calls and
// dd arithmetic on the host; only their dd products move to the GPU.
//
// pddblas's mulmm/mulltmm are not virtual; vcp::matrix<T, P> derives from P
// and calls this->mulmm(...), which name lookup resolves to the members
// below.  The slice count is a process-wide setting:
//     vcp::pddcuda_settings::slices() = 0;   // default: 13 (w = 104 bits)
// Non-zero statuses become vcp::dimension_error (bad shapes) or
// vcp::state_error, as pddblas reports its failures (vcp/error.hpp).
#ifndef VCP_CUDA_PDDCUDA_HPP
#define VCP_CUDA_PDDCUDA_HPP

#include <cmath>
#include <limits>
#include <vector>

#include <kv/dd.hpp>
#include <vcp/error.hpp>
#include <vcp/pddblas.hpp>

#include "../vcpcuda.h"

namespace vcp {

struct pddcuda_settings {
  static int& slices() {
    static int s = 0;
    return s;
  }
};
namespace pddcuda_detail {
inline int& slices_setting() { return pddcuda_settings::slices(); }
}  // namespace pddcuda_detail

namespace pddcuda_detail {
static_assert(sizeof(kv::dd) == 2 * sizeof(double), "kv::dd must be two packed doubles {a1, a2}");
inline const double* cd(const std::vector<kv::dd>& v) {
  return reinterpret_cast<const double*>(v.data());
}
inline double* md(std::vector<kv::dd>& v) { return reinterpret_cast<double*>(v.data()); }
inline void check(int st, const char* what) {
  if (st == VCPCU_OK) return;
  if (st == VCPCU_ERR_INVALID_ARG)
    vcp::throw_error<vcp::dimension_error>(what, ": ", vcpcu_last_error_string());
  vcp::throw_error<vcp::state_error>(what, ": ", vcpcu_last_error_string());
}
inline int& slices_setting();
// C (m x n) = op(A) B in dd on the GPU; op(A) = A (m x k) or, with transA,
// the transpose of A stored k x m (the two uses of pddblas_assist::ozaki_acc).
inline void dd_prod(const std::vector<kv::dd>& A, bool transA, const std::vector<kv::dd>& B,
                    int m, int n, int k, std::vector<kv::dd>& C) {
  std::vector<kv::dd> At;
  const std::vector<kv::dd>* a = &A;
  if (transA) {
    At.resize((size_t)m * k);
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < k; ++i) At[j + (size_t)m * i] = A[i + (size_t)k * j];
    a = &At;
  }
  C.assign((size_t)m * n, kv::dd(0.0));
  check(vcpcu_ddgemm(m, n, k, cd(*a), cd(B), md(C), nullptr, slices_setting()), "pddcuda");
}
}  // namespace pddcuda_detail

class pddcuda : public vcp::pddblas {
 public:
  // C = A * B (pddblas::mulmm): the scalar shortcuts and the result type
  // rules of pddblas, the product on the GPU.
  void mulmm(const pddcuda& B, pddcuda& c) const {
    if (this->type == 'S' || B.type == 'S') {
      vcp::pddblas::mulmm(B, c);
      return;
    }
    char ctype;
    if (this->type == 'R' && B.type == 'C' && this->column == B.row)
      ctype = 'S';
    else if (this->type == 'C' && B.type == 'R')
      ctype = 'M';
    else if (this->type == 'M' && B.type == 'C' && this->column == B.row)
      ctype = 'C';
    else if (this->type == 'R' && B.type == 'M' && this->column == B.row)
      ctype = 'R';
    else if (this->type == 'M' && B.type == 'M' && this->column == B.row)
      ctype = 'M';
    else {
      vcp::throw_error<vcp::dimension_error>("pddcuda::mulmm: unsupported matrix product: type ",
                                             this->type, " * ", B.type, ", size (", this->row,
                                             ", ", this->column, ") * (", B.row, ", ", B.column,
                                             ")");
      return;
    }
    const int m = this->row, k = this->column, nc = B.column;
    std::vector<kv::dd> Cv(m * nc);
    pddcuda_detail::check(vcpcu_ddgemm(m, nc, k, pddcuda_detail::cd(this->v),
                                       pddcuda_detail::cd(B.v), pddcuda_detail::md(Cv), nullptr,
                                       pddcuda_settings::slices()),
                          "pddcuda::mulmm");
    c.row = m;
    c.column = nc;
    c.n = m * nc;
    c.type = ctype;
    c.v = std::move(Cv);
  }

  // C = A^T A (pddblas::mulltmm), mirrored to exact symmetry as pddblas does.
  void mulltmm(pddcuda& c) const {
    if (this->type == 'S') {
      vcp::pddblas::mulltmm(c);
      return;
    }
    if (this->type != 'C' && this->type != 'R' && this->type != 'M')
      vcp::throw_error<vcp::state_error>("pddcuda::mulltmm: unsupported matrix type: ",
                                         this->type);
    const int m = this->row, nc = this->column;
    std::vector<kv::dd> At(this->v.size());
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < nc; ++j) At[j + nc * i] = this->v[i + m * j];
    std::vector<kv::dd> Cv(nc * nc);
    pddcuda_detail::check(vcpcu_ddgemm(nc, nc, m, pddcuda_detail::cd(At),
                                       pddcuda_detail::cd(this->v), pddcuda_detail::md(Cv),
                                       nullptr, pddcuda_settings::slices()),
                          "pddcuda::mulltmm");
    c.row = nc;
    c.column = nc;
    c.n = nc * nc;
    c.type = (nc == 1) ? 'S' : 'M';
    c.v = std::move(Cv);
    for (int i = 0; i < nc; i++)
      for (int j = i + 1; j < nc; j++) c.v[j + nc * i] = c.v[i + nc * j];
  }

  // A x = b (pddblas::linearsolve, vcp/pddblas.hpp:413-474): LU of double(A)
  // (dgetrf), then up to 10 corrections d = LU \ double(r), x += d, with the
  // residual r = b - A x in dd from the GPU product; stops at dd accuracy or
  // when the correction stagnates, as pddblas does.
  void linearsolve(vcp::pddblas& b, vcp::pddblas& x) {
    if (this->row != this->column || b.row != this->row)
      vcp::throw_error<vcp::dimension_error>("linearsolve: invalid dimensions: A=(", this->row,
                                             ", ", this->column, "), b=(", b.row, ", ",
                                             b.column, ")");
    using std::fabs;
    const int an = this->row, nrhs = b.column, nb = an * nrhs;
    vcp::pdblas Ad;
    dd_to_d(*this, Ad);
    std::vector<int> ipiv(an);
    int N = an, NRHS = nrhs, lda = an, ldb = an, info;
    dgetrf_(&N, &N, &Ad.v.front(), &lda, ipiv.data(), &info);
    if (info != 0) throw vcp::lapack_error("dgetrf", info, "linearsolve: dgetrf failed");
    x.zeros(an, nrhs);
    std::vector<kv::dd> r = b.v, Ax;
    vcp::pdblas rd;
    rd.zeros(an, nrhs);
    char TN[] = "N";
    double prev = std::numeric_limits<double>::infinity();
    for (int it = 0; it < 10; it++) {
      for (int i = 0; i < nb; i++) rd.v[i] = r[i].a1;
      dgetrs_(TN, &N, &NRHS, &Ad.v.front(), &lda, ipiv.data(), &rd.v.front(), &ldb, &info);
      if (info != 0) throw vcp::lapack_error("dgetrs", info, "linearsolve: dgetrs failed");
      double normd = 0.0, normx = 0.0;
      for (int i = 0; i < nb; i++) {
        x.v[i] += kv::dd(rd.v[i]);
        if (fabs(rd.v[i]) > normd) normd = fabs(rd.v[i]);
        if (fabs(x.v[i].a1) > normx) normx = fabs(x.v[i].a1);
      }
      if (normd == 0.0 || normd <= 0.25e-32 * normx || normd >= 0.5 * prev) break;
      prev = normd;
      pddcuda_detail::dd_prod(this->v, false, x.v, an, nrhs, an, Ax);
      for (int i = 0; i < nb; i++) r[i] = b.v[i] - Ax[i];
    }
  }

  // A = inv(A): A X = I by the linear solve above (pddblas::inv).
  void inv() override {
    if (this->row != this->column)
      vcp::throw_error<vcp::dimension_error>("inv: matrix must be square: ", this->row, " != ",
                                             this->column);
    vcp::pddblas b, x;
    b.eye(this->row);
    this->linearsolve(b, x);
    this->v = std::move(x.v);
  }

  // Upper Cholesky factor (pddblas::Cholesky, vcp/pddblas.hpp:490-563):
  // dpotrf in double, then two refinements U += W U with E = A - U^T U in dd
  // (GPU), G = U^-T E U^-1 in double (dtrsm), W = triu(G, 1) + diag(G) / 2.
  void Cholesky() override {
    if (!this->is_symmetric())
      vcp::throw_error<vcp::domain_error>("Cholesky: matrix must be symmetric");
    const int an = this->row, nn = an * an;
    vcp::pdblas Ud;
    dd_to_d(*this, Ud);
    Ud.Cholesky();
    std::vector<kv::dd> U(nn), E, F, W(nn);
    for (int i = 0; i < nn; i++) U[i] = kv::dd(Ud.v[i]);
    char cL[] = "L", cR[] = "R", cU[] = "U", cT[] = "T", cN[] = "N";
    double one = 1.0;
    int N = an;
    for (int it = 0; it < 2; it++) {
      pddcuda_detail::dd_prod(U, true, U, an, an, an, E);
      for (int i = 0; i < nn; i++) E[i] = this->v[i] - E[i];
      for (int i = 0; i < nn; i++) Ud.v[i] = U[i].a1;
      vcp::pdblas G;
      G.zeros(an, an);
      for (int i = 0; i < nn; i++) G.v[i] = E[i].a1;
      dtrsm_(cL, cU, cT, cN, &N, &N, &one, &Ud.v.front(), &N, &G.v.front(), &N);
      dtrsm_(cR, cU, cN, cN, &N, &N, &one, &Ud.v.front(), &N, &G.v.front(), &N);
      for (int j = 0; j < an; j++)
        for (int i = 0; i < an; i++) {
          double g = G.v[i + an * j];
          if (i > j) g = 0.0;
          else if (i == j) g *= 0.5;
          W[i + an * j] = kv::dd(g);
        }
      pddcuda_detail::dd_prod(W, false, U, an, an, an, F);
      for (int i = 0; i < nn; i++) U[i] += F[i];
    }
    for (int j = 0; j < an; j++)
      for (int i = j + 1; i < an; i++) U[i + an * j] = kv::dd(0.0);
    this->v = std::move(U);
  }

  // Symmetric / generalized symmetric eigenproblems (pddblas::eigsym,
  // eigsymge, vcp/pddblas.hpp:566-657): LAPACK dsyev / dsygv in double, then
  // at least two Ogita-Aishima steps with their dd products on the GPU.
  void eigsym(int itep = 4) override {
    vcp::pddblas V;
    this->eigsym(V, itep);
  }
  void eigsym(vcp::pddblas& V, int itep = 4) { refine_eig(nullptr, V, itep); }
  void eigsymge(vcp::pddblas& B, int itep = 1) {
    vcp::pddblas V;
    this->eigsymge(B, V, itep);
  }
  void eigsymge(vcp::pddblas& B, vcp::pddblas& V, int itep = 1) {
    if (!B.is_symmetric())
      vcp::throw_error<vcp::domain_error>("eigsymge: matrix B must be symmetric");
    if (this->row != B.row || this->column != B.column)
      vcp::throw_error<vcp::dimension_error>("eigsymge: dimension mismatch: A=(", this->row, ", ",
                                             this->column, "), B=(", B.row, ", ", B.column, ")");
    refine_eig(&B, V, itep);
  }

 private:
  void refine_eig(vcp::pddblas* B, vcp::pddblas& V, int itep) {
    if (!this->is_symmetric())
      vcp::throw_error<vcp::domain_error>(B ? "eigsymge: matrix A must be symmetric"
                                            : "eigsym: matrix must be symmetric");
    const int an = this->row, nn = an * an;
    vcp::pdblas Ad, Vd;
    dd_to_d(*this, Ad);
    if (B) {
      vcp::pdblas Bd;
      dd_to_d(*B, Bd);
      Ad.eigsymge(Bd, Vd);
    } else {
      Ad.eigsym(Vd);
    }
    std::vector<kv::dd> X(nn), lam(an);
    for (int i = 0; i < nn; i++) X[i] = kv::dd(Vd.v[i]);
    for (int i = 0; i < an; i++) lam[i] = kv::dd(Ad.v[i + an * i]);
    for (int it = 0; it < (itep < 2 ? 2 : itep); it++) oa_step_gpu(B, X, lam, an);
    V.zeros(an, an);
    V.v = std::move(X);
    this->zeros(an, an);
    for (int i = 0; i < an; i++) this->v[i + an * i] = lam[i];
  }

  // One Ogita-Aishima refinement of (X, lam) (pddblas::oa_step,
  // vcp/pddblas.hpp:221-314; T. Ogita, K. Aishima, JJIAM 2018): S = X^T A X,
  // G = X^T B X, lam_i = S_ii / G_ii, R = I - G, E from S, R and the
  // eigenvalue gaps (threshold delta), X += X E -- the four or five dd
  // products on the GPU.
  void oa_step_gpu(const vcp::pddblas* B, std::vector<kv::dd>& X, std::vector<kv::dd>& lam,
                   int n) const {
    using std::fabs;
    const int nn = n * n;
    std::vector<kv::dd> AX, S, G, BX, E(nn), XE;
    pddcuda_detail::dd_prod(this->v, false, X, n, n, n, AX);
    pddcuda_detail::dd_prod(X, true, AX, n, n, n, S);
    if (B) {
      pddcuda_detail::dd_prod(B->v, false, X, n, n, n, BX);
      pddcuda_detail::dd_prod(X, true, BX, n, n, n, G);
    } else {
      pddcuda_detail::dd_prod(X, true, X, n, n, n, G);
    }
    for (int i = 0; i < n; i++) lam[i] = S[i + n * i] / G[i + n * i];
    std::vector<kv::dd>& R = G;  // R = I - G
    for (int t = 0; t < nn; t++) R[t] = -R[t];
    for (int i = 0; i < n; i++) R[i + n * i] += kv::dd(1.0);
    double normR = 0.0, offS = 0.0, lmax = 0.0;
    for (int i = 0; i < n; i++) {
      double s1 = 0.0, s2 = 0.0;
      for (int j = 0; j < n; j++) {
        s1 += fabs(R[i + n * j].a1);
        if (i != j) s2 += fabs(S[i + n * j].a1);
      }
      if (s1 > normR) normR = s1;
      if (s2 > offS) offS = s2;
      if (fabs(lam[i].a1) > lmax) lmax = fabs(lam[i].a1);
    }
    const double delta = 2.0 * (offS + normR * lmax);
    const kv::dd half(0.5);
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        const kv::dd d = lam[j] - lam[i];
        E[i + n * j] = (i != j && fabs(d.a1) > delta)
                           ? (S[i + n * j] + lam[j] * R[i + n * j]) / d
                           : R[i + n * j] * half;
      }
    pddcuda_detail::dd_prod(X, false, E, n, n, n, XE);
    for (int t = 0; t < nn; t++) X[t] += XE[t];
  }
};

}  // namespace vcp

#endif  // VCP_CUDA_PDDCUDA_HPP
