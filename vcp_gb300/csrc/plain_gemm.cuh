// plain_gemm.cuh -- launchers of the FP64 directed-rounding kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

namespace vcpcu {

enum PointKind { PK_NEAREST = 0, PK_UP = 1, PK_DOWN = 2, PK_UPDOWN = 3 };

// C0 (and C1 for PK_UPDOWN, rounded down) = A * B, GEMM naming
// C(M x N) = A(M x K) B(K x N); K <= 0 zeroes the outputs.
int launch_point_gemm(int M, int N, int K, const double* A, long lda, const double* B,
                      long ldb, double* C0, double* C1, long ldc, int kind,
                      cudaStream_t s);

// Plain-form interval GEMM over kv-layout intervals; ws must hold
// interval_gemm_plain_ws_bytes(M, N, K) bytes.
int launch_interval_gemm_plain(int M, int N, int K, const double* A, long lda,
                               const double* B, long ldb, double* C, long ldc,
                               double* ws, cudaStream_t s);
size_t interval_gemm_plain_ws_bytes(int M, int N, int K);

// Thin right factor: products with N <= kThinN columns run in
// interval_gemm_thin_kernel (two lanes per row of C, no tile padding), with
// the same chains and results as the tile kernel.  a_point / b_point: A / B
// hold point entries (doubles, radius 0) instead of kv intervals.  ws holds
// interval_gemm_thin_ws_bytes(M, N, K, a_point) bytes (with an interval A:
// 32 bytes per entry of A for the operand pairs of the two lanes).
constexpr int kThinN = 16;
int launch_interval_gemm_thin(int M, int N, int K, const double* A, long lda, bool a_point,
                              const double* B, long ldb, bool b_point, double* C, long ldc,
                              double* ws, cudaStream_t s);
size_t interval_gemm_thin_ws_bytes(int M, int N, int K, bool a_point);

// R (M x N) = Y (M x K point) [C] (K x N kv) with imats::mul_m_im's loop
// (vcp/imats.hpp:203-213): kv interval products and sums term by term.
int launch_imats_mulmm(int M, int N, int K, const double* Y, long ldy, const double* C, long ldc,
                       double* R, long ldr, cudaStream_t s);

// C = [A]ᵀ[A] (A K x N interval) with pidblas::mulltmm semantics, full
// symmetric output; ws holds isyrk_plain_ws_bytes(N, K).
int launch_isyrk_plain(int N, int K, const double* A, long lda, double* C, long ldc, double* ws,
                       cudaStream_t s);
size_t isyrk_plain_ws_bytes(int N, int K);

}  // namespace vcpcu
