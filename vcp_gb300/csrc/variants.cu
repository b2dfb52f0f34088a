// variants.cu -- the other products on the interval GEMM path:
//   * interval x point and point x interval (pidblas::mul_im_m / mul_m_im,
//     vcp/pidblas.hpp:90-196): the point factor is widened to degenerate
//     intervals [b, b] (midrad gives b and radius +0 exactly), and the
//     interval GEMM of either form runs on them.  In the plain form the
//     extra radius chain is a chain of +0 products, so the result is
//     bit-identical to the three-dgemm formula of pidblas;
//   * [A]^T[A] (pidblas::mulltmm, vcp/pidblas.hpp:296-358) and the
//     verified A^T A of a point matrix (pidblas::vmulmm, :198-236);
//   * the upper bound of ||R [A] - I||_inf that imats::linearsolve checks
//     (vcp/imats.hpp:316-336 with mats::norminf, vcp/mats.hpp:1583-1597):
//     row sums of |.| accumulated upward in ascending column order, then the
//     largest row sum.
#include "common.cuh"
#include "ozaki.cuh"
#include "plain_gemm.cuh"
#include "variants.cuh"

namespace vcpcu {

namespace {

inline int grid1(long total) {
  long b = (total + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return b < 1 ? 1 : (int)b;
}

// point X (rows x cols, ldx) -> kv degenerate intervals (ld = rows)
__global__ void expand_point(int rows, int cols, const double* __restrict__ X, long ldx,
                             double* __restrict__ out) {
  long total = (long)rows * cols;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long i = idx % rows, j = idx / rows;
    const double v = X[i + j * ldx];
    out[2 * idx] = v;
    out[2 * idx + 1] = v;
  }
}

// point A (k x n, lda) -> Aᵀ (n x k, ld = n)
__global__ void transpose_point(int K, int N, const double* __restrict__ A, long lda,
                                double* __restrict__ At) {
  long total = (long)K * N;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long j = idx % N, p = idx / N;
    At[idx] = A[p + j * lda];
  }
}

// interval A (k x n, lda) -> Aᵀ (n x k, ld = n)
__global__ void transpose_iv(int K, int N, const double* __restrict__ A, long lda,
                             double* __restrict__ At) {
  long total = (long)K * N;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long j = idx % N, p = idx / N;
    const double* e = A + 2 * (p + j * lda);
    At[2 * idx] = e[0];
    At[2 * idx + 1] = e[1];
  }
}

// [CD, CU] planes (ld = n) -> kv intervals (ldc)
__global__ void pack_interval(int n, const double* __restrict__ CD, const double* __restrict__ CU,
                              double* __restrict__ C, long ldc) {
  long total = (long)n * n;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long i = idx % n, j = idx / n;
    C[2 * (i + j * ldc)] = CD[idx];
    C[2 * (i + j * ldc) + 1] = CU[idx];
  }
}

// mirror the upper triangle of a kv interval matrix into the lower one
__global__ void mirror_upper(int n, double* __restrict__ C, long ldc) {
  long total = (long)n * n;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long i = idx % n, j = idx / n;
    if (i > j) {
      C[2 * (i + j * ldc)] = C[2 * (j + i * ldc)];
      C[2 * (i + j * ldc) + 1] = C[2 * (j + i * ldc) + 1];
    }
  }
}

// Row sums of |RA - I| rounded upward, column order ascending (one thread per
// row; a warp reads 32 consecutive rows of one column).
__global__ void norm_rows(int n, const double* __restrict__ C, long ldc,
                          double* __restrict__ rows) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int j = 0; j < n; ++j) {
    double lo = C[2 * (i + (long)j * ldc)], up = C[2 * (i + (long)j * ldc) + 1];
    if (i == j) {
      lo = __dsub_rd(lo, 1.0);
      up = __dsub_ru(up, 1.0);
    }
    const double mg = fmax(fabs(lo), fabs(up));
    s = (j == 0) ? mg : __dadd_ru(s, mg);
  }
  rows[i] = s;
}

// largest entry (NaN propagates)
__global__ void max_of(int n, const double* __restrict__ v, double* __restrict__ out) {
  __shared__ double red[256];
  double m = -INFINITY;
  bool nan = false;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double x = v[i];
    if (isnan(x)) nan = true;
    m = fmax(m, x);
  }
  red[threadIdx.x] = nan ? __longlong_as_double(0x7ff8000000000000LL) : m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      const double a = red[threadIdx.x], b = red[threadIdx.x + w];
      red[threadIdx.x] = (isnan(a) || isnan(b)) ? __longlong_as_double(0x7ff8000000000000LL)
                                                : fmax(a, b);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

}  // namespace

int igemm_point_dispatch(int interval_side, int m, int n, int k, const double* L, long ldl,
                         const double* R, long ldr, double* C, long ldc, int form, int slices,
                         cudaStream_t s) {
  // widen the point factor into scratch, then the interval product
  const long prow = interval_side == 0 ? k : m, pcol = interval_side == 0 ? n : k;
  Scratch wide;
  int st = wide.alloc(sizeof(double) * 2 * (size_t)(prow > 0 ? prow : 1) * (pcol > 0 ? pcol : 1), s);
  if (st) return st;
  double* P = (double*)wide.ptr;
  if (prow > 0 && pcol > 0) {
    expand_point<<<grid1(prow * pcol), 256, 0, s>>>((int)prow, (int)pcol,
                                                      interval_side == 0 ? R : L,
                                                      interval_side == 0 ? ldr : ldl, P);
    VCPCU_LAUNCH_CHECK("expand_point");
  }
  if (interval_side == 0)
    return igemm_any(m, n, k, L, ldl, P, prow > 0 ? prow : 1, C, ldc, form, slices, s, 2);
  return igemm_any(m, n, k, P, prow > 0 ? prow : 1, R, ldr, C, ldc, form, slices, s, 1);
}

namespace {
// kv interval result (ld = rows) -> upper ends CU and lower ends CD (ldc)
__global__ void split_kv(int rows, int cols, const double* __restrict__ C, double* __restrict__ CU,
                         double* __restrict__ CD, long ldc) {
  long total = (long)rows * cols;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long i = idx % rows, j = idx / rows;
    const double2 c = reinterpret_cast<const double2*>(C)[idx];
    CD[i + j * ldc] = c.x;
    CU[i + j * ldc] = c.y;
  }
}
}  // namespace

int udmatmul_ozaki_dispatch(int m, int n, int k, const double* A, long lda, const double* B,
                            long ldb, double* CU, double* CD, long ldc, int slices,
                            cudaStream_t s) {
  // vblas naming: A m x n, B n x k, C m x k; as a BLAS product M = m, N = k, K = n
  if (n <= 0) {  // empty inner dimension: the exact product is 0
    VCPCU_CUDA_TRY(cudaMemset2DAsync(CU, sizeof(double) * ldc, 0, sizeof(double) * m, k, s));
    VCPCU_CUDA_TRY(cudaMemset2DAsync(CD, sizeof(double) * ldc, 0, sizeof(double) * m, k, s));
    return VCPCU_OK;
  }
  const size_t na = 2 * (size_t)m * (n > 0 ? n : 1), nb = 2 * (size_t)(n > 0 ? n : 1) * k,
               nc = 2 * (size_t)m * k;
  Scratch buf;
  int st = buf.alloc(sizeof(double) * (na + nb + nc), s);
  if (st) return st;
  double* PA = (double*)buf.ptr;
  double* PB = PA + na;
  double* PC = PB + nb;
  expand_point<<<grid1((long)m * n), 256, 0, s>>>(m, n, A, lda, PA);
  VCPCU_LAUNCH_CHECK("expand_point");
  expand_point<<<grid1((long)n * k), 256, 0, s>>>(n, k, B, ldb, PB);
  VCPCU_LAUNCH_CHECK("expand_point");
  if ((st = igemm_any(m, k, n, PA, m, PB, n, PC, m, VCPCU_FORM_OZAKI, slices, s, 3)))
    return st;
  split_kv<<<grid1((long)m * k), 256, 0, s>>>(m, k, PC, CU, CD, ldc);
  VCPCU_LAUNCH_CHECK("split_kv");
  return VCPCU_OK;
}

int isyrk_dispatch(int n, int k, const double* A, long lda, double* C, long ldc, int form,
                   int slices, cudaStream_t s) {
  if (form == VCPCU_FORM_PLAIN) {
    Scratch ws;
    int st = ws.alloc(isyrk_plain_ws_bytes(n, k > 0 ? k : 0) + 64, s);
    if (st) return st;
    return launch_isyrk_plain(n, k > 0 ? k : 0, A, lda, C, ldc, (double*)ws.ptr, s);
  }
  Scratch tr;
  int st = tr.alloc(sizeof(double) * 2 * (size_t)n * (k > 0 ? k : 1), s);
  if (st) return st;
  double* At = (double*)tr.ptr;
  if (k > 0) {
    transpose_iv<<<grid1((long)n * k), 256, 0, s>>>(k, n, A, lda, At);
    VCPCU_LAUNCH_CHECK("transpose_iv");
  }
  st = igemm_any(n, n, k, At, n, A, lda, C, ldc, form, slices, s);
  if (st) return st;
  mirror_upper<<<grid1((long)n * n), 256, 0, s>>>(n, C, ldc);
  VCPCU_LAUNCH_CHECK("mirror_upper");
  return VCPCU_OK;
}

int vsyrk_dispatch(int n, int k, const double* A, long lda, double* C, long ldc,
                   cudaStream_t s) {
  Scratch ws;
  const size_t nk = (size_t)n * (k > 0 ? k : 1), nn = (size_t)n * n;
  int st = ws.alloc(sizeof(double) * (nk + 2 * nn), s);
  if (st) return st;
  double* At = (double*)ws.ptr;
  double* CD = At + nk;
  double* CU = CD + nn;
  if (k > 0) {
    transpose_point<<<grid1((long)n * k), 256, 0, s>>>(k, n, A, lda, At);
    VCPCU_LAUNCH_CHECK("transpose_point");
  }
  // CU / CD (i,j) = chains of sum_p A(p,i) A(p,j): the dsyrk of vmulmm
  st = launch_point_gemm(n, n, k > 0 ? k : 0, At, n, A, lda, CU, CD, n, PK_UPDOWN, s);
  if (st) return st;
  pack_interval<<<grid1((long)n * n), 256, 0, s>>>(n, CD, CU, C, ldc);
  VCPCU_LAUNCH_CHECK("pack_interval");
  return VCPCU_OK;
}

int norm_dispatch(int n, const double* R, long ldr, const double* A, long lda, double* bound,
                  int form, int slices, cudaStream_t s) {
  Scratch ws;
  int st = ws.alloc(sizeof(double) * (2 * (size_t)n * n + n), s);
  if (st) return st;
  double* RA = (double*)ws.ptr;
  double* rows = RA + 2 * (size_t)n * n;
  st = igemm_point_dispatch(1, n, n, n, R, ldr, A, lda, RA, n, form, slices, s);
  if (st) return st;
  norm_rows<<<(n + 127) / 128, 128, 0, s>>>(n, RA, n, rows);
  VCPCU_LAUNCH_CHECK("norm_rows");
  max_of<<<1, 256, 0, s>>>(n, rows, bound);
  VCPCU_LAUNCH_CHECK("max_of");
  return VCPCU_OK;
}

}  // namespace vcpcu
