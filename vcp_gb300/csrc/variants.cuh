// variants.cuh -- interval x point, [A]^T[A], verified A^T A, ||R[A] - I||.
#pragma once
#include <cuda_runtime.h>

namespace vcpcu {

// VCPCU_FORM_PLAIN or VCPCU_FORM_OZAKI, whichever the cost model of the
// autotuner predicts faster (autotune.cu); batched: as one problem of a
// grouped batch (no per-product launch cost).
int autotune_choose(int m, int n, int k, bool batched = false);

// The AUTO decision for these operands (host or device pointers): the form
// of autotune_choose and, for the tensor-core form, the slice count whose
// enclosures the probe finds no wider than the plain form's (*slices = 0
// with *form = VCPCU_FORM_PLAIN when no candidate qualifies).
int autotune_pick(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                  cudaStream_t s, int* form, int* slices);

// Interval product of either form on device pointers (defined in capi.cu).
// point_mask bit 0 / bit 1: A / B has zero radii (the tensor-core form then
// skips the radius product that vanishes; the result is the same).
int igemm_any(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
              double* C, long ldc, int form, int slices, cudaStream_t s, int point_mask = 0);

// interval_side 0: C = [L] * R (R point, pidblas::mul_im_m);
// interval_side 1: C = L * [R] (L point, pidblas::mul_m_im).
int igemm_point_dispatch(int interval_side, int m, int n, int k, const double* L, long ldl,
                         const double* R, long ldr, double* C, long ldc, int form, int slices,
                         cudaStream_t s);
// CD <= A B <= CU by the tensor-core form (vblas naming: A m x n, B n x k).
int udmatmul_ozaki_dispatch(int m, int n, int k, const double* A, long lda, const double* B,
                            long ldb, double* CU, double* CD, long ldc, int slices,
                            cudaStream_t s);
int isyrk_dispatch(int n, int k, const double* A, long lda, double* C, long ldc, int form,
                   int slices, cudaStream_t s);
int vsyrk_dispatch(int n, int k, const double* A, long lda, double* C, long ldc, cudaStream_t s);
int norm_dispatch(int n, const double* R, long ldr, const double* A, long lda, double* bound,
                  int form, int slices, cudaStream_t s);

// The verification steps of imats::linearsolve given R and mx (variants.cu).
// The n^3 product R[A] runs in `form`; the three products with nrhs columns
// run in the plain form when nrhs <= kLssPlainRhs (FP64 thin kernel: faster
// there than padding nrhs to a 256-column tensor-core tile, and tighter).
constexpr int kLssPlainRhs = 4;

int ilss_thin_form(int form, int nrhs);
int ilss_verify_dispatch(int n, int nrhs, const double* A, long lda, const double* b, long ldb,
                         const double* R, long ldr, const double* mx, long ldmx, double* x,
                         long ldx, double* bound, int form, int slices, cudaStream_t s);

// The verification of imats::eigsymge in two device stages around the
// caller's inverse of mid(B X) (variants.cu); eig_merge_host is its final
// overlap merge.
int ieig_stage1_dispatch(int n, const double* A, long lda, const double* B, long ldb,
                         const double* X, long ldx, double* C, double* BX, double* M, int form,
                         int slices, cudaStream_t s);
int ieig_stage2_dispatch(int n, const double* lambda, const double* Y, long ldy, double* C,
                         const double* BX, double* lam, double* bound, int form, int slices,
                         cudaStream_t s);
void eig_merge_host(int n, double* lam);

// ifma.cu: elementwise inf-sup interval FMA and the ifma-chain product.
int launch_ifma(long count, const double* A, const double* B, const double* C, double* R,
                cudaStream_t s);
int launch_igemm_fma(int M, int N, int K, const double* A, long lda, const double* B, long ldb,
                     double* C, long ldc, cudaStream_t s);

}  // namespace vcpcu
