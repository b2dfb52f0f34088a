// vcp_cuda/pddcuda.hpp -- vcp::pddcuda, the GPU drop-in for vcp::pddblas.
//
// Use exactly like pddblas (vcp/pddblas.hpp:204):
//     vcp::matrix< kv::dd, vcp::pddcuda > A, B, C;
//     C = A * B;            // pddcuda::mulmm   (pddblas::mulmm,   pddblas.hpp:318)
//     C = ltransmul(A);     // pddcuda::mulltmm (pddblas::mulltmm, pddblas.hpp:379)
// The class derives from vcp::pddblas, so its solvers (linearsolve, eigsym,
// eigsymge) are inherited unchanged; the two products above are replaced by
// vcpcu_ddgemm (include/vcpcuda.h): the dd operands are scaled per row /
// column to w-bit integers, multiplied exactly on the tensor cores through
// residues modulo small primes, and rounded to the dd result -- the same
// product pddblas forms from error-free double slices, at least as accurate.
//
// pddblas's mulmm/mulltmm are not virtual; vcp::matrix<T, P> derives from P
// and calls this->mulmm(...), which name lookup resolves to the members
// below.  The slice count is a process-wide setting:
//     vcp::pddcuda_settings::slices() = 0;   // default: 13 (w = 104 bits)
// Non-zero statuses become vcp::dimension_error (bad shapes) or
// vcp::state_error, as pddblas reports its failures (vcp/error.hpp).
#ifndef VCP_CUDA_PDDCUDA_HPP
#define VCP_CUDA_PDDCUDA_HPP

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
};

}  // namespace vcp

#endif  // VCP_CUDA_PDDCUDA_HPP
