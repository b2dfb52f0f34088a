// vcp_cuda/pidcuda.hpp -- vcp::pidcuda, the GPU drop-in for vcp::pidblas.
//
// Use exactly like pidblas (vcp/pidblas.hpp:87):
//     vcp::matrix< kv::interval<double>, vcp::pidcuda > A, B, C;
//     C = A * B;                  // pidcuda::mulmm        (pidblas.hpp:239)
//     C = ltransmul(A);           // pidcuda::mulltmm      (pidblas.hpp:296)
//     x = lss(A, b);              // pidcuda::linearsolve -> vcpcu_ilss_verify
//     vcp::matrix< kv::interval<double>, vcp::pidcuda_fma > F;  // pidblas_fma drop-in
// The class derives from vcp::imats<double, vcp::pdblas> as pidblas does, so
// every imats algorithm (eigsym, ...) routes its interval products through
// the hooks below to libvcpcuda (include/vcpcuda.h); linearsolve and
// eigsymge are replaced by versions whose verification stays on the GPU.
//
// Form and precision are process-wide settings:
//     vcp::pidcuda_settings::form()   = VCPCU_FORM_OZAKI;   // default
//     vcp::pidcuda_settings::slices() = 0;                  // default precision
//     (+ VCPCU_SLICES_FAST_RADIUS: fewer radius GEMMs, see include/vcpcuda.h)
// VCPCU_FORM_PLAIN reproduces pidblas bit for bit over a sequential-chain
// BLAS; the Ozaki forms enclose the same products on the tensor cores.
// Non-zero statuses become vcp::dimension_error (bad shapes) or
// vcp::state_error (everything else), as pidblas reports its failures
// (vcp/error.hpp).  Scalar ('S') operands keep the host shortcuts of pidblas.
#ifndef VCP_CUDA_PIDCUDA_HPP
#define VCP_CUDA_PIDCUDA_HPP

#include <iostream>
#include <vector>

#include <kv/interval.hpp>
#include <vcp/error.hpp>
#include <vcp/imats.hpp>
#include <vcp/pdblas.hpp>

#include "../vcpcuda.h"

namespace vcp {

struct pidcuda_settings {
  static int& form() {
    static int f = VCPCU_FORM_OZAKI;
    return f;
  }
  static int& slices() {
    static int s = 0;
    return s;
  }
};

namespace pidcuda_detail {
static_assert(sizeof(kv::interval<double>) == 2 * sizeof(double),
              "kv::interval<double> must be two packed doubles {inf, sup}");
inline const double* cd(const std::vector<kv::interval<double> >& v) {
  return reinterpret_cast<const double*>(v.data());
}
inline double* md(std::vector<kv::interval<double> >& v) {
  return reinterpret_cast<double*>(v.data());
}
inline void check(int st, const char* what) {
  if (st == VCPCU_OK) return;
  if (st == VCPCU_ERR_INVALID_ARG)
    vcp::throw_error<vcp::dimension_error>(what, ": ", vcpcu_last_error_string());
  vcp::throw_error<vcp::state_error>(what, ": ", vcpcu_last_error_string());
}
// The inverse callback of vcpcu_ieigsymge: pdblas::inv (LAPACK) in place.
inline int pdblas_inverse(int n, double* M, void*) {
  try {
    vcp::pdblas Y;
    Y.zeros(n, n);
    for (long i = 0; i < (long)n * n; ++i) Y.v[i] = M[i];
    Y.inv();
    for (long i = 0; i < (long)n * n; ++i) M[i] = Y.v[i];
    return 0;
  } catch (...) {
    return 1;
  }
}
}  // namespace pidcuda_detail

class pidcuda : public vcp::imats<double, vcp::pdblas> {
  typedef vcp::imats<double, vcp::pdblas> base;

 protected:
  // C = [A] * B, B point (pidblas::mul_im_m)
  void mul_im_m(const vcp::pdblas& B, base& c) const override {
    if (this->type == 'S' || B.type == 'S') {
      base::mul_im_m(B, c);
      return;
    }
    if (this->column != B.row)
      vcp::throw_error<vcp::dimension_error>("pidcuda::mul_im_m: (", this->row, ", ",
                                             this->column, ") * (", B.row, ", ", B.column, ")");
    c.zeros(this->row, B.column);
    pidcuda_detail::check(
        vcpcu_igemm_point(0, this->row, B.column, this->column, pidcuda_detail::cd(this->v),
                          B.v.data(), pidcuda_detail::md(c.v), pidcuda_settings::form(),
                          pidcuda_settings::slices()),
        "pidcuda::mul_im_m");
  }
  // C = B * [A], B point (pidblas::mul_m_im)
  void mul_m_im(const vcp::pdblas& B, base& c) const override {
    if (this->type == 'S' || B.type == 'S') {
      base::mul_m_im(B, c);
      return;
    }
    if (B.column != this->row)
      vcp::throw_error<vcp::dimension_error>("pidcuda::mul_m_im: (", B.row, ", ", B.column,
                                             ") * (", this->row, ", ", this->column, ")");
    c.zeros(B.row, this->column);
    pidcuda_detail::check(
        vcpcu_igemm_point(1, B.row, this->column, B.column, B.v.data(),
                          pidcuda_detail::cd(this->v), pidcuda_detail::md(c.v),
                          pidcuda_settings::form(), pidcuda_settings::slices()),
        "pidcuda::mul_m_im");
  }
  // this = verified C^T C of a point C (pidblas::vmulmm)
  void vmulmm(const vcp::pdblas& C) override {
    if (C.type == 'S') {
      base::vmulmm(C);
      return;
    }
    this->zeros(C.column, C.column);
    pidcuda_detail::check(
        vcpcu_vsyrk(C.column, C.row, C.v.data(), pidcuda_detail::md(this->v)), "pidcuda::vmulmm");
  }

 public:
  // C = [A] * [B] (pidblas::mulmm)
  void mulmm(const vcp::mats<kv::interval<double> >& B,
             vcp::mats<kv::interval<double> >& c) const override {
    if (this->type == 'S' || B.type == 'S') {
      // scalar times matrix: elementwise interval products on the host
      if (this->type == 'S') {
        c = B;
        for (int i = 0; i < B.n; i++) c.v[i] *= this->v[0];
      } else {
        c = *this;
        for (int i = 0; i < this->n; i++) c.v[i] *= B.v[0];
      }
      return;
    }
    if (this->column != B.row)
      vcp::throw_error<vcp::dimension_error>("pidcuda::mulmm: (", this->row, ", ", this->column,
                                             ") * (", B.row, ", ", B.column, ")");
    c.zeros(this->row, B.column);
    pidcuda_detail::check(
        vcpcu_igemm(this->row, B.column, this->column, pidcuda_detail::cd(this->v),
                    pidcuda_detail::cd(B.v), pidcuda_detail::md(c.v), pidcuda_settings::form(),
                    pidcuda_settings::slices()),
        "pidcuda::mulmm");
  }
  // x = A \ b, verified (imats::linearsolve, vcp/imats.hpp:293-364).  R =
  // inv(mid A) and mx = R mid(b) are formed on the host as the reference
  // forms them (pdblas: LAPACK inverse, BLAS product); the verification --
  // four interval products, the norms and the enclosure -- runs on the GPU
  // in one call without host round trips (vcpcu_ilss_verify).  Found by
  // name from vcp::matrix's lss() (vcp/matrix.hpp:607-634) in place of the
  // base class's; n = 1 keeps the reference's scalar path.
  void linearsolve(base& b, base& x) {
    if (this->row != this->column || b.row != this->row)
      vcp::throw_error<vcp::dimension_error>("linearsolve: invalid dimensions: A=(", this->row,
                                             ", ", this->column, "), b=(", b.row, ", ",
                                             b.column, ")");
    if (this->row < 2) {
      base::linearsolve(b, x);
      return;
    }
    vcp::pdblas mx, mb, R;
    this->imid(R);
    mb.zeros(b.row, b.column);
    for (int i = 0; i < b.n; i++) mb.v[i] = mid(b.v[i]);
    R.inv();
    R.mulmm(mb, mx);
    mb.clear();
    x.zeros(b.row, b.column);
    double G = 0.0;
    const int st = vcpcu_ilss_verify(this->row, b.column, pidcuda_detail::cd(this->v),
                                     pidcuda_detail::cd(b.v), R.v.data(), mx.v.data(),
                                     pidcuda_detail::md(x.v), &G, pidcuda_settings::form(),
                                     pidcuda_settings::slices());
    if (st == VCPCU_OK || st == VCPCU_ERR_VERIFY)
      std::cout << "Linear solver Check || I - RA || < 1: " << G << " < 1 ?" << std::endl;
    if (st == VCPCU_ERR_VERIFY)
      vcp::throw_error<vcp::verification_error>("linearsolve verification failed: ||RA - I|| <= ",
                                                G);
    pidcuda_detail::check(st, "pidcuda::linearsolve");
  }
  // Enclosures of the eigenvalues of A x = lambda B x (imats::eigsymge,
  // vcp/imats.hpp:419-522; Miyajima's theorem).  The approximate eigenpairs
  // come from the host LAPACK as in the reference (pdblas::eigsymge), the
  // inverse of mid(B X) from pdblas::inv; the four interval products, the
  // norms and the enclosures run on the GPU (vcpcu_ieigsymge).  *this
  // becomes the diagonal matrix of the enclosures; n = 1 keeps the
  // reference's scalar path.
  void eigsymge(base& B, int itep = 1) {
    const int n = this->row;
    if (n < 2) {
      base::eigsymge(B, itep);
      return;
    }
    vcp::pdblas X, lambda;
    {
      vcp::pdblas mA, mB;
      this->imid(mA);
      mB.zeros(B.row, B.column);
      for (int i = 0; i < B.n; i++) mB.v[i] = mid(B.v[i]);
      mA.eigsymge(mB, X);
      mA.diag(lambda);
    }
    std::vector<double> lam(2 * (size_t)n);
    double bound = 0.0;
    const int st = vcpcu_ieigsymge(n, pidcuda_detail::cd(this->v), pidcuda_detail::cd(B.v),
                                   X.v.data(), lambda.v.data(), &pidcuda_detail::pdblas_inverse,
                                   nullptr, lam.data(), &bound, pidcuda_settings::form(),
                                   pidcuda_settings::slices());
    if (st == VCPCU_ERR_VERIFY)
      vcp::throw_error<vcp::verification_error>("eigsymge verification failed: ||YBX - I|| <= ",
                                                bound);
    pidcuda_detail::check(st, "pidcuda::eigsymge");
    this->zeros(n, n);
    for (int i = 0; i < n; i++)
      this->v[i + n * i] = kv::interval<double>(lam[2 * i], lam[2 * i + 1]);
  }
  // C = [A]^T [A] (pidblas::mulltmm)
  void mulltmm(vcp::mats<kv::interval<double> >& c) const override {
    if (this->type == 'S') {
      c.zeros(1, 1);
      c.v[0] = this->v[0] * this->v[0];
      return;
    }
    c.zeros(this->column, this->column);
    pidcuda_detail::check(
        vcpcu_isyrk(this->column, this->row, pidcuda_detail::cd(this->v), pidcuda_detail::md(c.v),
                    pidcuda_settings::form(), pidcuda_settings::slices()),
        "pidcuda::mulltmm");
  }
};

// vcp::pidcuda_fma -- the GPU drop-in for vcp::pidblas_fma
// (vcp/pidblas_fma.hpp:43-80): pidcuda with the interval product replaced by
// the inf-sup ifma chain (vcpcu_igemm_fma), bit-identical to pidblas_fma's
// loop; the other hooks stay those of pidcuda.
class pidcuda_fma : public pidcuda {
 public:
  void mulmm(const vcp::mats<kv::interval<double> >& B,
             vcp::mats<kv::interval<double> >& c) const override {
    if (this->type == 'S' || B.type == 'S') {
      pidcuda::mulmm(B, c);
      return;
    }
    if (this->column != B.row)
      vcp::throw_error<vcp::dimension_error>("pidcuda_fma::mulmm: (", this->row, ", ",
                                             this->column, ") * (", B.row, ", ", B.column, ")");
    c.zeros(this->row, B.column);
    pidcuda_detail::check(vcpcu_igemm_fma(this->row, B.column, this->column,
                                          pidcuda_detail::cd(this->v), pidcuda_detail::cd(B.v),
                                          pidcuda_detail::md(c.v)),
                          "pidcuda_fma::mulmm");
  }
};

}  // namespace vcp

#endif  // VCP_CUDA_PIDCUDA_HPP
