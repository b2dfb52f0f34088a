// ozaki.cu -- placeholder until the tensor-core form lands.
#include "common.cuh"
#include "ozaki.cuh"

namespace vcpcu {
int ozaki_igemm(int, int, int, const double*, long, const double*, long, double*, long, int,
                int, cudaStream_t) {
  set_error("igemm: the Ozaki form is not built yet");
  return VCPCU_ERR_UNSUPPORTED;
}
}  // namespace vcpcu
