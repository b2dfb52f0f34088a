// vcp_cuda/rmatmul_cuda.hpp -- vblas rmatmul / udmatmul on the GPU.
//
// Same signatures and semantics as vblas/rmatmul.hpp:102 and
// vblas/udmatmul.hpp:758 (column-major, A m x n, B n x k, C m x k; every
// entry the ascending sequential FMA chain rounded in the requested
// direction; the caller's rounding mode is never touched), so
//     #include <vcp_cuda/rmatmul_cuda.hpp>
//     vcp_cuda::rmatmul(m, n, k, A, B, CU, 1);
// replaces the vblas call, with bit-identical results.  Defining
// VCP_CUDA_VBLAS_NAMES before the include also provides the unqualified
// global names rmatmul / udmatmul (do not include vblas/rmatmul.hpp in the
// same translation unit then).  Failures throw std::runtime_error, as vblas
// does when no backend is available (vblas/rmatmul.hpp:90-96).
#ifndef VCP_CUDA_RMATMUL_CUDA_HPP
#define VCP_CUDA_RMATMUL_CUDA_HPP

#include <stdexcept>
#include <string>

#include "../vcpcuda.h"

namespace vcp_cuda {

inline void rmatmul(int m, int n, int k, const double* A, const double* B, double* CU,
                    const int rounding_mode) {
  const int st = vcpcu_rmatmul(m, n, k, A, B, CU, rounding_mode);
  if (st) throw std::runtime_error(std::string("vcpcu_rmatmul: ") + vcpcu_last_error_string());
}

inline void udmatmul(int m, int n, int k, double* A, double* B, double* CU, double* CD) {
  const int st = vcpcu_udmatmul(m, n, k, A, B, CU, CD);
  if (st) throw std::runtime_error(std::string("vcpcu_udmatmul: ") + vcpcu_last_error_string());
}

}  // namespace vcp_cuda

#ifdef VCP_CUDA_VBLAS_NAMES
inline void rmatmul(int m, int n, int k, const double* A, const double* B, double* CU,
                    const int rounding_mode) {
  vcp_cuda::rmatmul(m, n, k, A, B, CU, rounding_mode);
}
inline void udmatmul(int m, int n, int k, double* A, double* B, double* CU, double* CD) {
  vcp_cuda::udmatmul(m, n, k, A, B, CU, CD);
}
#endif

#endif  // VCP_CUDA_RMATMUL_CUDA_HPP
