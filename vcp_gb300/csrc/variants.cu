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
#include "swfp.cuh"
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

// The upper end of kv abs([lo, up]), on the integer pipe (swfp.cuh).
__device__ __forceinline__ double abs_sup(double lo, double up) { return sw_abs_sup(lo, up); }

// Row sums of |RA - I| rounded upward, column order ascending (one thread per
// row; a warp reads 32 consecutive rows of one column).  The sums are
// sequential chains, so there are only n threads: each keeps two groups of
// PF columns in flight ahead of its additions.
template <bool SHIFT = true>
__global__ void norm_rows(int n, const double* __restrict__ C, long ldc,
                          double* __restrict__ rows) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  constexpr int PF = 16;
  const double2* c2 = reinterpret_cast<const double2*>(C);
  auto load = [&](int j) -> double2 {
    return j < n ? c2[i + (long)j * ldc] : make_double2(0.0, 0.0);
  };
  double2 cur[PF], nxt[PF];
#pragma unroll
  for (int p = 0; p < PF; ++p) cur[p] = load(p);
  // the warp's rows i0 .. i0 + 31 meet the diagonal only in the column
  // groups that overlap them (a warp-uniform test): elsewhere no FP64
  // subtraction is issued, not even predicated off
  const int i0 = i & ~31;
  double s = 0.0;
  for (int jb = 0; jb < n; jb += PF) {
#pragma unroll
    for (int p = 0; p < PF; ++p) nxt[p] = load(jb + PF + p);
    if (!SHIFT || jb + PF <= i0 || jb >= i0 + 32) {
#pragma unroll
      for (int p = 0; p < PF; ++p) {
        const int j = jb + p;
        if (j < n) {
          const double mg = abs_sup(cur[p].x, cur[p].y);
          s = (j == 0) ? mg : __dadd_ru(s, mg);
        }
      }
    } else {
#pragma unroll
      for (int p = 0; p < PF; ++p) {
        const int j = jb + p;
        if (j < n) {
          double lo = cur[p].x, up = cur[p].y;
          if (i == j) {
            lo = __dsub_rd(lo, 1.0);
            up = __dsub_ru(up, 1.0);
          }
          const double mg = abs_sup(lo, up);
          s = (j == 0) ? mg : __dadd_ru(s, mg);
        }
      }
    }
#pragma unroll
    for (int p = 0; p < PF; ++p) cur[p] = nxt[p];
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
  const int f = form == VCPCU_FORM_AUTO ? autotune_choose(m, n, k) : form;
  if (f == VCPCU_FORM_PLAIN && n <= kThinN) {
    // thin plain product: the kernel reads the point factor as is
    if (m <= 0 || n <= 0) return VCPCU_OK;
    Scratch ws;
    int st = ws.alloc(interval_gemm_thin_ws_bytes(m, n, k, interval_side == 1), s);
    if (st) return st;
    return launch_interval_gemm_thin(m, n, k > 0 ? k : 0, L, ldl, interval_side == 1, R, ldr,
                                     interval_side == 0, C, ldc, (double*)ws.ptr, s);
  }
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

// ---------------------------------------------------------------------------
// The verification of imats::linearsolve (vcp/imats.hpp:293-364) after its
// approximate inverse R = inv(mid A) and approximate solution mx = R mid(b):
//   P = [A] mx - [b]                     (mul_im_m, subsmmA       :305-307)
//   r = R P                              (mul_m_im                :309)
//   E = R [A] - I, G = ||E||_inf         (mul_m_im, norminf       :317-329)
//   t = || |r| ||_inf, g = t / (1 - G)   (norminf, division       :336-345)
//   H = |E| (g ... g)                    (abs, mulmm              :341-353)
//   x = mx + [-u, u], u = |r| + H        (addmm, add_im_m         :355-363)
// with kv interval arithmetic step by step, so that the plain form gives
// the reference's bits.
namespace {

// P -= Q elementwise (kv interval subtraction), P rows x cols with ld = rows.
__global__ void iv_sub(int rows, int cols, double* __restrict__ P, const double* __restrict__ Q,
                       long ldq) {
  const long total = (long)rows * cols;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const long i = idx % rows, j = idx / rows;
    const double2 p = reinterpret_cast<const double2*>(P)[idx];
    const double* q = Q + 2 * (i + j * ldq);
    reinterpret_cast<double2*>(P)[idx] = make_double2(__dsub_rd(p.x, q[1]), __dsub_ru(p.y, q[0]));
  }
}

// Row values of mats::norminf (vcp/mats.hpp:1565-1600) for |r|: a matrix
// (rows, cols > 1) sums |r(i, j)| upward in ascending j; a vector or a scalar
// takes the largest |r| (std::max order) -- max_last then picks the largest
// row value as the reference's loop over rows does.
__global__ void mag_rows(int rows, int cols, const double* __restrict__ R, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (rows > 1 && cols == 1) {  // a column vector: one entry per row
    if (i < rows) out[i] = abs_sup(R[2 * (long)i], R[2 * (long)i + 1]);
    return;
  }
  if (i >= rows) return;
  const bool sum = rows > 1 && cols > 1;
  double s = 0.0;
  for (int j = 0; j < cols; ++j) {
    const double* e = R + 2 * (i + (long)j * rows);
    const double mg = abs_sup(e[0], e[1]);
    s = j == 0 ? mg : (sum ? __dadd_ru(s, mg) : (mg < s ? s : mg));
  }
  out[i] = s;
}

// c = v[0]; c = std::max(v[i], c) for i = 1..n-1 (kv max of the intervals'
// upper ends): the largest value, and of equal ones the last.  One block;
// the (value, index) reduction is order-independent.
__global__ void max_last(int n, const double* __restrict__ v, double* __restrict__ out) {
  __shared__ double rv[256];
  __shared__ int ri[256];
  double bv = v[0];
  int bi = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double x = v[i];
    if (!(x < bv) && (bv < x || i > bi)) {
      bv = x;
      bi = i;
    }
  }
  rv[threadIdx.x] = bv;
  ri[threadIdx.x] = bi;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      const double x = rv[threadIdx.x + w];
      const int xi = ri[threadIdx.x + w];
      const double y = rv[threadIdx.x];
      const int yi = ri[threadIdx.x];
      if (y < x || (!(x < y) && xi > yi)) {
        rv[threadIdx.x] = x;
        ri[threadIdx.x] = xi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = rv[0];
}

// g = [t, t] / (1 - [G, G]) by kv's interval division with both operands
// positive: [RD(t / RU(1 - G)), RU(t / RD(1 - G))]; then E -> |E| with the
// diagonal shifted (E = RA - I) is done by abs_shift, and H's factor
// (g ... g) by fill_iv.
__global__ void lss_scale(const double* __restrict__ G, const double* __restrict__ t,
                          double* __restrict__ g) {
  const double d_lo = __dsub_rd(1.0, *G), d_up = __dsub_ru(1.0, *G);
  const double tt = *t;
  const double q[4] = {__ddiv_rd(tt, d_lo), __ddiv_rd(tt, d_up), __ddiv_rd(tt, d_lo),
                       __ddiv_rd(tt, d_up)};
  const double u[4] = {__ddiv_ru(tt, d_lo), __ddiv_ru(tt, d_up), __ddiv_ru(tt, d_lo),
                       __ddiv_ru(tt, d_up)};
  double lo = q[0], up = u[0];  // std::min_element / max_element: the first extreme
  for (int c = 1; c < 4; ++c) {
    if (q[c] < lo) lo = q[c];
    if (up < u[c]) up = u[c];
  }
  g[0] = lo;
  g[1] = up;
}

// E(i, i) -= 1 (interval minus point; SHIFT), then E -> kv abs(E), in place.
template <bool SHIFT = true>
__global__ void abs_shift(int n, double* __restrict__ E) {
  const long total = (long)n * n;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const long i = idx % n, j = idx / n;
    double2 e = reinterpret_cast<const double2*>(E)[idx];
    if (SHIFT && i == j) {
      e.x = __dsub_rd(e.x, 1.0);
      e.y = __dsub_ru(e.y, 1.0);
    }
    double lo, up;
    sw_abs_iv(e.x, e.y, lo, up);
    reinterpret_cast<double2*>(E)[idx] = make_double2(lo, up);
  }
}

__global__ void fill_iv(long count, const double* __restrict__ g, double* __restrict__ T) {
  const double2 v = make_double2(g[0], g[1]);
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < count;
       idx += (long)gridDim.x * blockDim.x)
    reinterpret_cast<double2*>(T)[idx] = v;
}

// x = mx + [-u, u], u = RU(sup|r| + sup H) (addmm, the symmetric widening and
// add_im_m of vcp/imats.hpp:355-363).
__global__ void lss_final(int rows, int cols, const double* __restrict__ r,
                          const double* __restrict__ H, const double* __restrict__ mx, long ldmx,
                          double* __restrict__ x, long ldx) {
  const long total = (long)rows * cols;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const long i = idx % rows, j = idx / rows;
    const double u = __dadd_ru(abs_sup(r[2 * idx], r[2 * idx + 1]), H[2 * idx + 1]);
    const double m = mx[i + j * ldmx];
    x[2 * (i + j * ldx)] = __dadd_rd(-u, m);
    x[2 * (i + j * ldx) + 1] = __dadd_ru(u, m);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// The verification of imats::eigsymge (vcp/imats.hpp:419-522, Miyajima's
// eigenvalue enclosure for A x = lambda B x) around the caller's approximate
// eigenpairs (X, lambda) of the midpoints and its approximate inverse
// Y = inv(mid(B X)):
//   stage 1   C = [A] X, BX = [B] X (pidblas::mul_im_m, :430-435), mid(BX)
//   stage 2   C = C - BX (lambda ... lambda)              (:440-445)
//             R = Y C (the base class's kv loop, :448), Rinf = ||R||, Re = |R| e
//             S = Y BX - I (pidblas::mul_m_im, :458-462), Sinf = ||S||, Se = |S| e
//             g = Rinf / (1 - Sinf); lam = lambda + [-u, u], u = sup(Re + g Se)
// with kv's operation at every step.  In the plain form R = Y C runs the base
// class's term-by-term loop (imats_mulmm_kernel), so all bits are the
// reference's; the tensor-core form encloses it by the CRT product.
namespace {

// kv midpoints of an interval matrix (count entries), integer pipe.
__global__ void mid_of(long count, const double* __restrict__ X, double* __restrict__ M) {
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < count;
       idx += (long)gridDim.x * blockDim.x) {
    const double2 e = reinterpret_cast<const double2*>(X)[idx];
    double m, r, p;
    sw_midrad(e.x, e.y, m, r, p);
    M[idx] = m;
  }
}

// kv's product of intervals x * y: the first smallest of the four round-down
// products and the first largest of the four round-up ones (std::min_element
// / max_element over x.inf y.inf, x.inf y.sup, x.sup y.inf, x.sup y.sup).
__device__ __forceinline__ void kv_mul_iv(double xl, double xu, double yl, double yu, double& lo,
                                          double& up) {
  const double a[4] = {__dmul_rd(xl, yl), __dmul_rd(xl, yu), __dmul_rd(xu, yl),
                       __dmul_rd(xu, yu)};
  const double b[4] = {__dmul_ru(xl, yl), __dmul_ru(xl, yu), __dmul_ru(xu, yl),
                       __dmul_ru(xu, yu)};
  lo = a[0];
  up = b[0];
#pragma unroll
  for (int c = 1; c < 4; ++c) {
    if (a[c] < lo) lo = a[c];
    if (up < b[c]) up = b[c];
  }
}

// C(i, j) -= BX(i, j) * [lambda_j, lambda_j] (kv product, kv subtraction).
__global__ void sub_lambda(int n, double* __restrict__ C, const double* __restrict__ BX,
                           const double* __restrict__ lambda) {
  const long total = (long)n * n;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const double l = lambda[idx / n];
    const double2 b = reinterpret_cast<const double2*>(BX)[idx];
    const double2 c = reinterpret_cast<const double2*>(C)[idx];
    // [l, l] is the second factor: x.inf y.inf, x.inf y.sup, x.sup y.inf, ...
    const double p1 = __dmul_rd(b.x, l), p3 = __dmul_rd(b.y, l);
    const double q1 = __dmul_ru(b.x, l), q3 = __dmul_ru(b.y, l);
    const double pl = p3 < p1 ? p3 : p1, pu = q1 < q3 ? q3 : q1;
    reinterpret_cast<double2*>(C)[idx] = make_double2(__dsub_rd(c.x, pu), __dsub_ru(c.y, pl));
  }
}

// imats::mul_im_m 'M' x 'C' with the ones vector (vcp/imats.hpp:88-97): per row
// c = X(i, 0), then c = X(i, j) + c outward, j ascending.
__global__ void iv_row_sums(int n, const double* __restrict__ X, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  constexpr int PF = 16;
  const double2* x2 = reinterpret_cast<const double2*>(X);
  auto load = [&](int j) -> double2 { return j < n ? x2[i + (long)j * n] : make_double2(0.0, 0.0); };
  double2 cur[PF], nxt[PF];
#pragma unroll
  for (int p = 0; p < PF; ++p) cur[p] = load(p);
  double lo = 0.0, up = 0.0;
  for (int jb = 0; jb < n; jb += PF) {
#pragma unroll
    for (int p = 0; p < PF; ++p) nxt[p] = load(jb + PF + p);
#pragma unroll
    for (int p = 0; p < PF; ++p) {
      const int j = jb + p;
      if (j < n) {
        lo = j == 0 ? cur[p].x : __dadd_rd(cur[p].x, lo);
        up = j == 0 ? cur[p].y : __dadd_ru(cur[p].y, up);
      }
    }
#pragma unroll
    for (int p = 0; p < PF; ++p) cur[p] = nxt[p];
  }
  out[2 * i] = lo;
  out[2 * i + 1] = up;
}

// lam_i = lambda_i + [-u, u], u = RU(sup Re_i + sup(g * Se_i)) (mulsm, addmm and
// the symmetric widening of vcp/imats.hpp:488-499); g = sc[0..1].
__global__ void eig_final(int n, const double* __restrict__ Re, const double* __restrict__ Se,
                          const double* __restrict__ g, const double* __restrict__ lambda,
                          double* __restrict__ lam) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double sl, su;
  kv_mul_iv(g[0], g[1], Se[2 * i], Se[2 * i + 1], sl, su);
  const double u = __dadd_ru(Re[2 * i + 1], su);
  lam[2 * i] = __dadd_rd(-u, lambda[i]);
  lam[2 * i + 1] = __dadd_ru(u, lambda[i]);
}

}  // namespace

int ieig_stage1_dispatch(int n, const double* A, long lda, const double* B, long ldb,
                         const double* X, long ldx, double* C, double* BX, double* M, int form,
                         int slices, cudaStream_t s) {
  int st;
  if ((st = igemm_point_dispatch(0, n, n, n, A, lda, X, ldx, C, n, form, slices, s))) return st;
  if ((st = igemm_point_dispatch(0, n, n, n, B, ldb, X, ldx, BX, n, form, slices, s))) return st;
  mid_of<<<grid1((long)n * n), 256, 0, s>>>((long)n * n, BX, M);
  VCPCU_LAUNCH_CHECK("mid_of");
  return VCPCU_OK;
}

int ieig_stage2_dispatch(int n, const double* lambda, const double* Y, long ldy, double* C,
                         const double* BX, double* lam, double* bound, int form, int slices,
                         cudaStream_t s) {
  const size_t nn = 2 * (size_t)n * n;
  Scratch ws;
  int st = ws.alloc(sizeof(double) * (nn + 5 * (size_t)n + 8), s);
  if (st) return st;
  double* P = (double*)ws.ptr;  // R, then S
  double* Re = P + nn;
  double* Se = Re + 2 * n;
  double* rows = Se + 2 * n;
  double* sc = rows + n;  // Rinf, g_lo, g_up
  sub_lambda<<<grid1((long)n * n), 256, 0, s>>>(n, C, BX, lambda);
  VCPCU_LAUNCH_CHECK("sub_lambda");
  if (form == VCPCU_FORM_PLAIN)
    st = launch_imats_mulmm(n, n, n, Y, ldy, C, n, P, n, s);
  else
    st = igemm_point_dispatch(1, n, n, n, Y, ldy, C, n, P, n, form, slices, s);
  if (st) return st;
  norm_rows<false><<<(n + 127) / 128, 128, 0, s>>>(n, P, n, rows);
  VCPCU_LAUNCH_CHECK("norm_rows");
  max_last<<<1, 256, 0, s>>>(n, rows, sc);
  VCPCU_LAUNCH_CHECK("max_last");
  abs_shift<false><<<grid1((long)n * n), 256, 0, s>>>(n, P);
  VCPCU_LAUNCH_CHECK("abs_shift");
  iv_row_sums<<<(n + 127) / 128, 128, 0, s>>>(n, P, Re);
  VCPCU_LAUNCH_CHECK("iv_row_sums");
  if ((st = igemm_point_dispatch(1, n, n, n, Y, ldy, BX, n, P, n, form, slices, s))) return st;
  norm_rows<true><<<(n + 127) / 128, 128, 0, s>>>(n, P, n, rows);
  VCPCU_LAUNCH_CHECK("norm_rows");
  max_last<<<1, 256, 0, s>>>(n, rows, bound);
  VCPCU_LAUNCH_CHECK("max_last");
  abs_shift<true><<<grid1((long)n * n), 256, 0, s>>>(n, P);
  VCPCU_LAUNCH_CHECK("abs_shift");
  iv_row_sums<<<(n + 127) / 128, 128, 0, s>>>(n, P, Se);
  VCPCU_LAUNCH_CHECK("iv_row_sums");
  lss_scale<<<1, 1, 0, s>>>(bound, sc, sc + 1);  // g = [Rinf, Rinf] / (1 - [Sinf, Sinf])
  VCPCU_LAUNCH_CHECK("lss_scale");
  eig_final<<<(n + 127) / 128, 128, 0, s>>>(n, Re, Se, sc + 1, lambda, lam);
  VCPCU_LAUNCH_CHECK("eig_final");
  return VCPCU_OK;
}

// The overlap merge of imats::eigsymge (vcp/imats.hpp:502-519), on the host.
void eig_merge_host(int n, double* lam) {
  for (int i = 0; i < n; ++i) {
    int j = 0;
    for (;;) {
      if (i != j) {
        double* x = lam + 2 * i;
        double* y = lam + 2 * j;
        const bool ov = x[0] <= y[1] && y[0] <= x[1];
        if (ov && (x[0] != y[0] || x[1] != y[1])) {
          x[0] = y[0] < x[0] ? y[0] : x[0];
          x[1] = x[1] < y[1] ? y[1] : x[1];
          y[0] = x[0];
          y[1] = x[1];
          j = 0;
          continue;
        }
      }
      if (++j == n) break;
    }
  }
}

int ilss_thin_form(int form, int nrhs) {
  return (form == VCPCU_FORM_PLAIN || nrhs <= kLssPlainRhs) ? VCPCU_FORM_PLAIN : form;
}

int ilss_verify_dispatch(int n, int nrhs, const double* A, long lda, const double* b, long ldb,
                         const double* R, long ldr, const double* mx, long ldmx, double* x,
                         long ldx, double* bound, int form, int slices, cudaStream_t s) {
  const size_t nv = 2 * (size_t)n * nrhs, nn = 2 * (size_t)n * n;
  Scratch ws;
  int st = ws.alloc(sizeof(double) * (nn + 4 * nv + n + 4), s);
  if (st) return st;
  double* E = (double*)ws.ptr;  // R[A] - I, then |R[A] - I|
  double* P = E + nn;
  double* r = P + nv;
  double* T = r + nv;
  double* H = T + nv;
  double* rows = H + nv;
  double* sc = rows + n;  // t, g_lo, g_up
  const int tf = ilss_thin_form(form, nrhs);
  if ((st = igemm_point_dispatch(0, n, nrhs, n, A, lda, mx, ldmx, P, n, tf, slices, s))) return st;
  iv_sub<<<grid1((long)n * nrhs), 256, 0, s>>>(n, nrhs, P, b, ldb);
  VCPCU_LAUNCH_CHECK("iv_sub");
  if ((st = igemm_point_dispatch(1, n, nrhs, n, R, ldr, P, n, r, n, tf, slices, s))) return st;
  if ((st = igemm_point_dispatch(1, n, n, n, R, ldr, A, lda, E, n, form, slices, s))) return st;
  norm_rows<<<(n + 127) / 128, 128, 0, s>>>(n, E, n, rows);
  VCPCU_LAUNCH_CHECK("norm_rows");
  max_of<<<1, 256, 0, s>>>(n, rows, bound);
  VCPCU_LAUNCH_CHECK("max_of");
  mag_rows<<<(n + 127) / 128, 128, 0, s>>>(n, nrhs, r, rows);
  VCPCU_LAUNCH_CHECK("mag_rows");
  max_last<<<1, 256, 0, s>>>(n, rows, sc);
  VCPCU_LAUNCH_CHECK("max_last");
  lss_scale<<<1, 1, 0, s>>>(bound, sc, sc + 1);
  VCPCU_LAUNCH_CHECK("lss_scale");
  abs_shift<<<grid1((long)n * n), 256, 0, s>>>(n, E);
  VCPCU_LAUNCH_CHECK("abs_shift");
  fill_iv<<<grid1((long)n * nrhs), 256, 0, s>>>((long)n * nrhs, sc + 1, T);
  VCPCU_LAUNCH_CHECK("fill_iv");
  if ((st = igemm_any(n, nrhs, n, E, n, T, n, H, n, tf, slices, s))) return st;
  lss_final<<<grid1((long)n * nrhs), 256, 0, s>>>(n, nrhs, r, H, mx, ldmx, x, ldx);
  VCPCU_LAUNCH_CHECK("lss_final");
  return VCPCU_OK;
}

}  // namespace vcpcu
