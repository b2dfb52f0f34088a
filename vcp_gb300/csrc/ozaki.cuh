// ozaki.cuh -- Ozaki-scheme interval GEMM on tcgen05 tensor cores.
#pragma once
#include <cuda_runtime.h>

namespace vcpcu {

constexpr int OZ_MAX_SLICES = 12;

int ozaki_igemm(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                double* C, long ldc, int form, int slices, cudaStream_t s);

}  // namespace vcpcu
