// capi.cu -- the exported C ABI (include/vcpcuda.h): argument checks,
// host<->device staging for the host-pointer entry points, dispatch.
#include <vector>

#include "common.cuh"
#include "plain_gemm.cuh"
#include "ozaki.cuh"
#include "variants.cuh"

#include <cstdlib>
#include <cstring>

using namespace vcpcu;

namespace {

// Non-blocking streams per (host thread, device) for the host-pointer entry
// points, so they do not serialise with unrelated work: 0 computes, 1 and 2
// carry the host->device and device->host copies of a pipelined product, 3
// and 4 its block products.
cudaStream_t host_stream(int which = 0) {
  thread_local cudaStream_t streams[64][5] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || which < 0 || which > 4) return nullptr;
  if (!streams[dev][which]) cudaStreamCreateWithFlags(&streams[dev][which], cudaStreamNonBlocking);
  return streams[dev][which];
}

// Blocks of a pipelined host-pointer product: column panels
// VCPCU_HOST_PANELS if set (1 with one row panel turns the pipeline off),
// else one per 1024 columns, at most 4; row panels VCPCU_HOST_ROW_PANELS if
// set, else one per 2048 rows, at most 4.  Products narrower than 2048
// columns run in one piece.  Measured end to end at n = 8192: 4 x 4 blocks
// 25.8 ms, 4 x 2 26.0, 2 x 2 26.9, 4 x 1 28.0 (copies at about 200 GB/s each
// way); n = 4096: 4 x 2 5.25 ms, 4 x 1 5.6.
int env_int(const char* name) {
  const char* v = getenv(name);
  return v ? atoi(v) : 0;
}
int host_panels(int n) {
  const int env = env_int("VCPCU_HOST_PANELS");
  if (env > 0) return env;
  if (n < 2048) return 1;
  return n / 1024 < 4 ? n / 1024 : 4;
}
// Row blocks of about 1365 rows, at most 6 (n = 8192: 6 x 4 blocks, 25.27 ms
// end to end against 25.61 for 4 x 4 on one box; more column blocks were
// slower).
int host_row_panels(int m, int n) {
  const int env = env_int("VCPCU_HOST_ROW_PANELS");
  if (env > 0) return env;
  if (n < 2048) return 1;
  const int r = m / 1365;
  return r < 1 ? 1 : (r > 6 ? 6 : r);
}

int point_kind(int rounding_mode) {
  if (rounding_mode == 1) return PK_UP;
  if (rounding_mode == -1) return PK_DOWN;
  return PK_NEAREST;
}

// vblas naming -> GEMM naming: rmatmul(m, n, k): A m x n, B n x k, C m x k.
int rmatmul_dev_impl(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                     double* C0, double* C1, int ldc, int kind, cudaStream_t s) {
  clear_error();
  if (m <= 0 || k <= 0) return VCPCU_OK;
  if (!C0 || (kind == PK_UPDOWN && !C1)) {
    set_error("rmatmul: null output pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (ldc < m) {
    set_error("rmatmul: ldc (%d) < m (%d)", ldc, m);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (n > 0) {
    if (!A || !B) {
      set_error("rmatmul: null input pointer");
      return VCPCU_ERR_INVALID_ARG;
    }
    if (lda < m || ldb < n) {
      set_error("rmatmul: lda (%d) < m (%d) or ldb (%d) < n (%d)", lda, m, ldb, n);
      return VCPCU_ERR_INVALID_ARG;
    }
  }
  int st = check_device();
  if (st) return st;
  return launch_point_gemm(m, k, n > 0 ? n : 0, A, lda, B, ldb, C0, C1, ldc, kind, s);
}

int rmatmul_host_impl(int m, int n, int k, const double* A, const double* B, double* C0,
                      double* C1, int kind) {
  clear_error();
  if (m <= 0 || k <= 0) return VCPCU_OK;
  if (!C0 || (kind == PK_UPDOWN && !C1) || (n > 0 && (!A || !B))) {
    set_error("rmatmul: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  cudaStream_t s = host_stream();
  const size_t na = n > 0 ? (size_t)m * n : 0, nb = n > 0 ? (size_t)n * k : 0,
               nc = (size_t)m * k;
  const size_t nouts = (kind == PK_UPDOWN) ? 2 : 1;
  Scratch buf;
  st = buf.alloc(sizeof(double) * (na + nb + nouts * nc), s);
  if (st) return st;
  double* dA = (double*)buf.ptr;
  double* dB = dA + na;
  double* dC0 = dB + nb;
  double* dC1 = (kind == PK_UPDOWN) ? dC0 + nc : nullptr;
  if (na) VCPCU_CUDA_TRY(cudaMemcpyAsync(dA, A, na * sizeof(double), cudaMemcpyHostToDevice, s));
  if (nb) VCPCU_CUDA_TRY(cudaMemcpyAsync(dB, B, nb * sizeof(double), cudaMemcpyHostToDevice, s));
  st = launch_point_gemm(m, k, n > 0 ? n : 0, dA, m, dB, n > 0 ? n : 1, dC0, dC1, m, kind, s);
  if (st) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(C0, dC0, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (dC1) VCPCU_CUDA_TRY(cudaMemcpyAsync(C1, dC1, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return VCPCU_OK;
}

int igemm_check(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                const double* C, int ldc, int form, int slices) {
  if (form != VCPCU_FORM_PLAIN && form != VCPCU_FORM_OZAKI && form != VCPCU_FORM_AUTO &&
      form != VCPCU_FORM_OZAKI_SLICES) {
    set_error("igemm: unknown form %d", form);
    return VCPCU_ERR_INVALID_ARG;
  }
  const int sc = oz_slice_count(slices);
  if ((form == VCPCU_FORM_OZAKI || form == VCPCU_FORM_OZAKI_SLICES) && sc != 0 &&
      (sc < 2 || sc > OZ_MAX_SLICES)) {
    set_error("igemm: slices must be 0 or in [2, %d] (optionally + VCPCU_SLICES_FAST_RADIUS), "
              "got %d", OZ_MAX_SLICES, slices);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (!C || (k > 0 && (!A || !B))) {
    set_error("igemm: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (ldc < m || (k > 0 && (lda < m || ldb < k))) {
    set_error("igemm: leading dimension too small (lda %d, ldb %d, ldc %d for m %d, k %d)", lda,
              ldb, ldc, m, k);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (form != VCPCU_FORM_PLAIN && k > 0 &&
      (((uintptr_t)A | (uintptr_t)B) & 15) != 0) {
    set_error("igemm: the Ozaki form reads intervals as 16-byte pairs; A and B must be "
              "16-byte aligned");
    return VCPCU_ERR_INVALID_ARG;
  }
  return VCPCU_OK;
}

}  // namespace

int vcpcu::igemm_any(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                     double* C, long ldc, int form, int slices, cudaStream_t s, int point_mask) {
  if (k < 0) k = 0;
  if (form == VCPCU_FORM_AUTO) {
    if (k > 0 && ((((uintptr_t)A) | ((uintptr_t)B)) & 15) != 0) {
      form = VCPCU_FORM_PLAIN;  // the tensor-core form reads 16-byte pairs
    } else {
      int st = autotune_pick(m, n, k, A, lda, B, ldb, s, &form, &slices);
      if (st) return st;
    }
  }
  if (form == VCPCU_FORM_PLAIN) {
    Scratch ws;
    int st = ws.alloc(interval_gemm_plain_ws_bytes(m, n, k), s);
    if (st) return st;
    return launch_interval_gemm_plain(m, n, k, A, lda, B, ldb, C, ldc, (double*)ws.ptr, s);
  }
  return ozaki_igemm(m, n, k, A, lda, B, ldb, C, ldc, form, slices, s, point_mask);
}

namespace {

int igemm_dispatch(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                   double* C, long ldc, int form, int slices, cudaStream_t s) {
  return igemm_any(m, n, k, A, lda, B, ldb, C, ldc, form, slices, s);
}

int form_check(int form, int slices) {
  if (form != VCPCU_FORM_PLAIN && form != VCPCU_FORM_OZAKI && form != VCPCU_FORM_AUTO &&
      form != VCPCU_FORM_OZAKI_SLICES) {
    set_error("unknown form %d", form);
    return VCPCU_ERR_INVALID_ARG;
  }
  const int sc = oz_slice_count(slices);
  if (form != VCPCU_FORM_PLAIN && sc != 0 && (sc < 2 || sc > OZ_MAX_SLICES)) {
    set_error("slices must be 0 or in [2, %d] (optionally + VCPCU_SLICES_FAST_RADIUS), got %d",
              OZ_MAX_SLICES, slices);
    return VCPCU_ERR_INVALID_ARG;
  }
  return VCPCU_OK;
}

bool misaligned16(const void* p) { return ((uintptr_t)p & 15) != 0; }

// Copies `n` doubles host -> device into dst (skips n == 0).
int h2d(double* dst, const double* src, size_t n, cudaStream_t s) {
  if (n) VCPCU_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, s));
  return VCPCU_OK;
}

int take_status() {
  int status = 0;
  int st = oz_take_status(host_stream(), &status);
  if (st) return st;
  if (status & 2) {
    set_error("igemm (Ozaki form): a bounded device-side wait timed out; result invalid");
    return VCPCU_ERR_TIMEOUT;
  }
  if (status & 1) {
    set_error("igemm (Ozaki form): non-finite input entry; the result is NaN");
    return VCPCU_ERR_NONFINITE;
  }
  return VCPCU_OK;
}

}  // namespace

extern "C" {

int vcpcu_status(void* stream) {
  clear_error();
  int status = 0;
  int st = oz_take_status((cudaStream_t)stream, &status);
  if (st) return st;
  if (status & 2) {
    set_error("a bounded device-side wait timed out in an earlier call");
    return VCPCU_ERR_TIMEOUT;
  }
  if (status & 1) {
    set_error("an earlier Ozaki-form call saw a non-finite input (its result is NaN)");
    return VCPCU_ERR_NONFINITE;
  }
  return VCPCU_OK;
}

int vcpcu_selftest_timeout(long long limit_cycles, void* stream) {
  clear_error();
  int st = check_device();
  if (st) return st;
  if (limit_cycles <= 0) limit_cycles = 2000000000LL;
  if (limit_cycles > 8000000000LL) {
    set_error("selftest_timeout: limit above 8e9 cycles");
    return VCPCU_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if ((st = oz_selftest_timeout(limit_cycles, s))) return st;
  return vcpcu_status(stream);
}

int vcpcu_profile(int enable) { return oz_profile_enable(enable); }

int vcpcu_profile_read(double* ms, int nphases, long long* tensor_flops) {
  return oz_profile_read(ms, nphases, tensor_flops);
}

int vcpcu_rmatmul(int m, int n, int k, const double* A, const double* B, double* C,
                  int rounding_mode) {
  return rmatmul_host_impl(m, n, k, A, B, C, nullptr, point_kind(rounding_mode));
}

int vcpcu_udmatmul(int m, int n, int k, const double* A, const double* B, double* CU,
                   double* CD) {
  return rmatmul_host_impl(m, n, k, A, B, CU, CD, PK_UPDOWN);
}

int vcpcu_rmatmul_dev(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                      double* C, int ldc, int rounding_mode, void* stream) {
  return rmatmul_dev_impl(m, n, k, A, lda, B, ldb, C, nullptr, ldc, point_kind(rounding_mode),
                          (cudaStream_t)stream);
}

int vcpcu_udmatmul_dev(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                       double* CU, double* CD, int ldc, void* stream) {
  return rmatmul_dev_impl(m, n, k, A, lda, B, ldb, CU, CD, ldc, PK_UPDOWN, (cudaStream_t)stream);
}

int vcpcu_ifma_dev(long count, const double* A, const double* B, const double* C, double* R,
                   void* stream) {
  clear_error();
  if (count <= 0) return VCPCU_OK;
  if (!A || !B || !C || !R) {
    set_error("ifma: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (misaligned16(A) || misaligned16(B)) {
    set_error("ifma: A and B must be 16-byte aligned");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  return launch_ifma(count, A, B, C, R, (cudaStream_t)stream);
}

int vcpcu_ifma(long count, const double* A, const double* B, const double* C, double* R) {
  clear_error();
  if (count <= 0) return VCPCU_OK;
  if (!A || !B || !C || !R) {
    set_error("ifma: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  cudaStream_t s = host_stream();
  const size_t n2 = 2 * (size_t)count;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * 4 * n2, s))) return st;
  double* dA = (double*)buf.ptr;
  double* dB = dA + n2;
  double* dC = dB + n2;
  double* dR = dC + n2;
  if ((st = h2d(dA, A, n2, s)) || (st = h2d(dB, B, n2, s)) || (st = h2d(dC, C, n2, s))) return st;
  if ((st = launch_ifma(count, dA, dB, dC, dR, s))) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(R, dR, n2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return VCPCU_OK;
}

int vcpcu_igemm_fma_dev(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                        double* C, int ldc, void* stream) {
  clear_error();
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && (!A || !B)) || ldc < m || (k > 0 && (lda < m || ldb < k))) {
    set_error("igemm_fma: null pointer or leading dimension too small");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (k > 0 && (misaligned16(A) || misaligned16(B))) {
    set_error("igemm_fma: A and B must be 16-byte aligned");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  return launch_igemm_fma(m, n, k, A, lda, B, ldb, C, ldc, (cudaStream_t)stream);
}

int vcpcu_igemm_fma(int m, int n, int k, const double* A, const double* B, double* C) {
  clear_error();
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && (!A || !B))) {
    set_error("igemm_fma: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  cudaStream_t s = host_stream();
  const size_t na = 2 * (size_t)m * k, nb = 2 * (size_t)k * n, nc = 2 * (size_t)m * n;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * (na + nb + nc), s))) return st;
  double* dA = (double*)buf.ptr;
  double* dB = dA + na;
  double* dC = dB + nb;
  if ((st = h2d(dA, A, na, s)) || (st = h2d(dB, B, nb, s))) return st;
  if ((st = launch_igemm_fma(m, n, k, dA, m, dB, k > 0 ? k : 1, dC, m, s))) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(C, dC, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return VCPCU_OK;
}

namespace {
int udoz_check(int m, int n, int k, const void* A, const void* B, const void* CU, const void* CD,
               int slices) {
  if (slices != 0 && (slices < 2 || slices > OZ_MAX_SLICES)) {
    set_error("udmatmul_ozaki: slices must be 0 or in [2, %d], got %d", OZ_MAX_SLICES, slices);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (m <= 0 || k <= 0) return VCPCU_OK;
  if (!CU || !CD || (n > 0 && (!A || !B))) {
    set_error("udmatmul_ozaki: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  return VCPCU_OK;
}
}  // namespace

int vcpcu_udmatmul_ozaki_dev(int m, int n, int k, const double* A, int lda, const double* B,
                             int ldb, double* CU, double* CD, int ldc, int slices, void* stream) {
  clear_error();
  int st = udoz_check(m, n, k, A, B, CU, CD, slices);
  if (st || m <= 0 || k <= 0) return st;
  if (n < 0) n = 0;
  if (ldc < m || (n > 0 && (lda < m || ldb < n))) {
    set_error("udmatmul_ozaki: leading dimension too small (lda %d, ldb %d, ldc %d)", lda, ldb,
              ldc);
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  return udmatmul_ozaki_dispatch(m, n, k, A, lda, B, ldb, CU, CD, ldc, slices,
                                 (cudaStream_t)stream);
}

int vcpcu_udmatmul_ozaki(int m, int n, int k, const double* A, const double* B, double* CU,
                         double* CD, int slices) {
  clear_error();
  int st = udoz_check(m, n, k, A, B, CU, CD, slices);
  if (st || m <= 0 || k <= 0) return st;
  if (n < 0) n = 0;
  if ((st = check_device())) return st;
  cudaStream_t s = host_stream();
  const size_t na = (size_t)m * n, nb = (size_t)n * k, nc = (size_t)m * k;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * (na + nb + 2 * nc), s))) return st;
  double* dA = (double*)buf.ptr;
  double* dB = dA + na;
  double* dU = dB + nb;
  double* dD = dU + nc;
  if ((st = h2d(dA, A, na, s)) || (st = h2d(dB, B, nb, s))) return st;
  st = udmatmul_ozaki_dispatch(m, n, k, dA, m, dB, n > 0 ? n : 1, dU, dD, m, slices, s);
  if (st) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(CU, dU, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaMemcpyAsync(CD, dD, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return take_status();
}

int vcpcu_igemm_dev(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                    double* C, int ldc, int form, int slices, void* stream) {
  clear_error();
  int st = igemm_check(m, n, k, A, lda, B, ldb, C, ldc, form, slices);
  if (st || m <= 0 || n <= 0) return st;
  st = check_device();
  if (st) return st;
  return igemm_dispatch(m, n, k, A, lda, B, ldb, C, ldc, form, slices, (cudaStream_t)stream);
}

int vcpcu_igemm(int m, int n, int k, const double* A, const double* B, double* C, int form,
                int slices) {
  clear_error();
  int st = igemm_check(m, n, k, A, m, B, k > 0 ? k : 1, C, m, form, slices);
  if (st || m <= 0 || n <= 0) return st;
  st = check_device();
  if (st) return st;
  if (k < 0) k = 0;
  cudaStream_t s = host_stream();
  int resolved = form;
  if (form == VCPCU_FORM_AUTO) {
    if (k > 0 && ((((uintptr_t)A) | ((uintptr_t)B)) & 15) != 0) {
      resolved = VCPCU_FORM_PLAIN;
    } else {
      st = autotune_pick(m, n, k, A, m, B, k, s, &resolved, &slices);
      if (st) return st;
    }
    form = resolved;
  }
  const int panels = host_panels(n), row_panels = host_row_panels(m, n);
  if (resolved == VCPCU_FORM_OZAKI && panels * row_panels > 1) {
    st = ozaki_igemm_host_pipelined(m, n, k, A, B, C, slices, panels, row_panels, s,
                                    host_stream(3), host_stream(4), host_stream(1),
                                    host_stream(2));
    if (st) return st;
    return take_status();
  }
  const size_t na = 2 * (size_t)m * k, nb = 2 * (size_t)k * n, nc = 2 * (size_t)m * n;
  Scratch buf;
  st = buf.alloc(sizeof(double) * (na + nb + nc), s);
  if (st) return st;
  double* dA = (double*)buf.ptr;
  double* dB = dA + na;
  double* dC = dB + nb;
  if (na) VCPCU_CUDA_TRY(cudaMemcpyAsync(dA, A, na * sizeof(double), cudaMemcpyHostToDevice, s));
  if (nb) VCPCU_CUDA_TRY(cudaMemcpyAsync(dB, B, nb * sizeof(double), cudaMemcpyHostToDevice, s));
  st = igemm_dispatch(m, n, k, dA, m, dB, k > 0 ? k : 1, dC, m, form, slices, s);
  if (st) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(C, dC, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  if (form != VCPCU_FORM_PLAIN) return take_status();
  return VCPCU_OK;
}

int vcpcu_igemm_point_dev(int interval_side, int m, int n, int k, const double* L, int ldl,
                          const double* R, int ldr, double* C, int ldc, int form, int slices,
                          void* stream) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (interval_side != 0 && interval_side != 1) {
    set_error("igemm_point: interval_side must be 0 ([L]*R) or 1 (L*[R])");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && (!L || !R)) || ldc < m || (k > 0 && (ldl < m || ldr < k))) {
    set_error("igemm_point: null pointer or leading dimension too small");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (form != VCPCU_FORM_PLAIN && k > 0 && misaligned16(interval_side == 0 ? L : R)) {
    set_error("igemm_point: the interval factor must be 16-byte aligned for the Ozaki form");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  return igemm_point_dispatch(interval_side, m, n, k, L, ldl, R, ldr, C, ldc, form, slices,
                              (cudaStream_t)stream);
}

int vcpcu_igemm_point(int interval_side, int m, int n, int k, const double* L, const double* R,
                      double* C, int form, int slices) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (interval_side != 0 && interval_side != 1) {
    set_error("igemm_point: interval_side must be 0 ([L]*R) or 1 (L*[R])");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && (!L || !R))) {
    set_error("igemm_point: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  cudaStream_t s = host_stream();
  const size_t wl = interval_side == 0 ? 2 : 1, wr = interval_side == 0 ? 1 : 2;
  const size_t nl = wl * (size_t)m * k, nr = wr * (size_t)k * n, nc = 2 * (size_t)m * n;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * (nl + nr + nc), s))) return st;
  // the interval factor first, so that it is 16-byte aligned
  double* base = (double*)buf.ptr;
  double* dL = interval_side == 0 ? base : base + nr;
  double* dR = interval_side == 0 ? base + nl : base;
  double* dC = base + nl + nr;
  if ((st = h2d(dL, L, nl, s)) || (st = h2d(dR, R, nr, s))) return st;
  st = igemm_point_dispatch(interval_side, m, n, k, dL, m, dR, k > 0 ? k : 1, dC, m, form, slices,
                            s);
  if (st) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(C, dC, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return form != VCPCU_FORM_PLAIN ? take_status() : VCPCU_OK;
}

int vcpcu_isyrk_dev(int n, int k, const double* A, int lda, double* C, int ldc, int form,
                    int slices, void* stream) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && !A) || ldc < n || (k > 0 && lda < k)) {
    set_error("isyrk: null pointer or leading dimension too small");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  return isyrk_dispatch(n, k, A, lda, C, ldc, form, slices, (cudaStream_t)stream);
}

int vcpcu_isyrk(int n, int k, const double* A, double* C, int form, int slices) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && !A)) {
    set_error("isyrk: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  cudaStream_t s = host_stream();
  const size_t na = 2 * (size_t)k * n, nc = 2 * (size_t)n * n;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * (na + nc), s))) return st;
  double* dA = (double*)buf.ptr;
  double* dC = dA + na;
  if ((st = h2d(dA, A, na, s))) return st;
  if ((st = isyrk_dispatch(n, k, dA, k > 0 ? k : 1, dC, n, form, slices, s))) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(C, dC, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return form != VCPCU_FORM_PLAIN ? take_status() : VCPCU_OK;
}

int vcpcu_vsyrk_dev(int n, int k, const double* A, int lda, double* C, int ldc, void* stream) {
  clear_error();
  if (n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && !A) || ldc < n || (k > 0 && lda < k)) {
    set_error("vsyrk: null pointer or leading dimension too small");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  return vsyrk_dispatch(n, k, A, lda, C, ldc, (cudaStream_t)stream);
}

int vcpcu_vsyrk(int n, int k, const double* A, double* C) {
  clear_error();
  if (n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && !A)) {
    set_error("vsyrk: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  cudaStream_t s = host_stream();
  const size_t na = (size_t)k * n, nc = 2 * (size_t)n * n;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * (na + nc), s))) return st;
  double* dA = (double*)buf.ptr;
  double* dC = dA + na;
  if ((st = h2d(dA, A, na, s))) return st;
  if ((st = vsyrk_dispatch(n, k, dA, k > 0 ? k : 1, dC, n, s))) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(C, dC, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return VCPCU_OK;
}

int vcpcu_norm_I_minus_RA_dev(int n, const double* R, int ldr, const double* A, int lda,
                              double* bound, int form, int slices, void* stream) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0 || !R || !A || !bound || ldr < n || lda < n) {
    set_error("norm_I_minus_RA: n must be positive, pointers non-null, ld >= n");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (form != VCPCU_FORM_PLAIN && misaligned16(A)) {
    set_error("norm_I_minus_RA: A must be 16-byte aligned for the Ozaki form");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  return norm_dispatch(n, R, ldr, A, lda, bound, form, slices, (cudaStream_t)stream);
}

int vcpcu_norm_I_minus_RA(int n, const double* R, const double* A, double* bound, int form,
                          int slices) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0 || !R || !A || !bound) {
    set_error("norm_I_minus_RA: n must be positive and pointers non-null");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  cudaStream_t s = host_stream();
  const size_t nr = (size_t)n * n, na = 2 * (size_t)n * n;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * (nr + na + 1), s))) return st;
  double* dA = (double*)buf.ptr;  // interval factor first: 16-byte aligned
  double* dR = dA + na;
  double* dB = dR + nr;
  if ((st = h2d(dR, R, nr, s)) || (st = h2d(dA, A, na, s))) return st;
  if ((st = norm_dispatch(n, dR, n, dA, n, dB, form, slices, s))) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(bound, dB, sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return form != VCPCU_FORM_PLAIN ? take_status() : VCPCU_OK;
}

int vcpcu_ilss_verify_dev(int n, int nrhs, const double* A, int lda, const double* b, int ldb,
                          const double* R, int ldr, const double* mx, int ldmx, double* x,
                          int ldx, double* bound, int form, int slices, void* stream) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0 || nrhs <= 0 || !A || !b || !R || !mx || !x || !bound || lda < n || ldb < n ||
      ldr < n || ldmx < n || ldx < n) {
    set_error("ilss_verify: n, nrhs must be positive, pointers non-null, ld >= n");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (form != VCPCU_FORM_PLAIN && (misaligned16(A) || misaligned16(b))) {
    set_error("ilss_verify: A and b must be 16-byte aligned for the Ozaki form");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  return ilss_verify_dispatch(n, nrhs, A, lda, b, ldb, R, ldr, mx, ldmx, x, ldx, bound, form,
                              slices, (cudaStream_t)stream);
}

int vcpcu_ilss_verify(int n, int nrhs, const double* A, const double* b, const double* R,
                      const double* mx, double* x, double* bound, int form, int slices) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0 || nrhs <= 0 || !A || !b || !R || !mx || !x || !bound) {
    set_error("ilss_verify: n, nrhs must be positive and pointers non-null");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  cudaStream_t s = host_stream();
  const size_t na = 2 * (size_t)n * n, nv = 2 * (size_t)n * nrhs, nr = (size_t)n * n,
               nm = (size_t)n * nrhs;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * (na + 2 * nv + nr + nm + 2), s))) return st;
  double* dA = (double*)buf.ptr;  // interval arrays first: 16-byte aligned
  double* db = dA + na;
  double* dx = db + nv;
  double* dR = dx + nv;
  double* dm = dR + nr;
  double* dG = dm + nm;
  if ((st = h2d(dA, A, na, s)) || (st = h2d(db, b, nv, s)) || (st = h2d(dR, R, nr, s)) ||
      (st = h2d(dm, mx, nm, s)))
    return st;
  if ((st = ilss_verify_dispatch(n, nrhs, dA, n, db, n, dR, n, dm, n, dx, n, dG, form, slices, s)))
    return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(x, dx, nv * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaMemcpyAsync(bound, dG, sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  if (form != VCPCU_FORM_PLAIN && (st = take_status())) return st;
  if (*bound >= 1.0) {
    set_error("ilss_verify: ||RA - I|| <= %.17g is not below 1", *bound);
    return VCPCU_ERR_VERIFY;
  }
  return VCPCU_OK;
}

int vcpcu_ieigsymge_stage1_dev(int n, const double* A, int lda, const double* B, int ldb,
                               const double* X, int ldx, double* C, double* BX, double* midBX,
                               int form, int slices, void* stream) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0 || !A || !B || !X || !C || !BX || !midBX || lda < n || ldb < n || ldx < n) {
    set_error("ieigsymge: n must be positive, pointers non-null, ld >= n");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (misaligned16(C) || misaligned16(BX) ||
      (form != VCPCU_FORM_PLAIN && (misaligned16(A) || misaligned16(B)))) {
    set_error("ieigsymge: interval arrays must be 16-byte aligned");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  return ieig_stage1_dispatch(n, A, lda, B, ldb, X, ldx, C, BX, midBX, form, slices,
                              (cudaStream_t)stream);
}

int vcpcu_ieigsymge_stage2_dev(int n, const double* lambda, const double* Y, int ldy, double* C,
                               const double* BX, double* lam, double* bound, int form,
                               int slices, void* stream) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0 || !lambda || !Y || !C || !BX || !lam || !bound || ldy < n) {
    set_error("ieigsymge: n must be positive, pointers non-null, ldy >= n");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (misaligned16(C) || misaligned16(BX) || misaligned16(lam)) {
    set_error("ieigsymge: interval arrays must be 16-byte aligned");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  return ieig_stage2_dispatch(n, lambda, Y, ldy, C, BX, lam, bound, form, slices,
                              (cudaStream_t)stream);
}

int vcpcu_eig_merge(int n, double* lam) {
  clear_error();
  if (n < 0 || (n > 0 && !lam)) {
    set_error("eig_merge: n must be non-negative and lam non-null");
    return VCPCU_ERR_INVALID_ARG;
  }
  eig_merge_host(n, lam);
  return VCPCU_OK;
}

int vcpcu_ieigsymge(int n, const double* A, const double* B, const double* X,
                    const double* lambda, vcpcu_inverse_fn inv, void* ctx, double* lam,
                    double* bound, int form, int slices) {
  clear_error();
  int st = form_check(form, slices);
  if (st) return st;
  if (n <= 0 || !A || !B || !X || !lambda || !inv || !lam || !bound) {
    set_error("ieigsymge: n must be positive and pointers non-null");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  cudaStream_t s = host_stream();
  const size_t nn = (size_t)n * n;
  // interval arrays first (16-byte aligned): A, B, C, BX (2 nn each), lam (2 n);
  // then X, mid(BX) / Y (nn each), lambda (n), the bound (1)
  const size_t oB = 2 * nn, oC = 4 * nn, oBX = 6 * nn, oLam = 8 * nn, oX = oLam + 2 * (size_t)n,
               oM = oX + nn, oL = oM + nn, oG = oL + n, total = oG + 1;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * total, s))) return st;
  double* dA = (double*)buf.ptr;
  double* dB = dA + oB;
  double* dC = dA + oC;
  double* dBX = dA + oBX;
  double* dlam = dA + oLam;
  double* dX = dA + oX;
  double* dM = dA + oM;  // mid(BX), then Y
  double* dl = dA + oL;
  double* dG = dA + oG;
  if ((st = h2d(dA, A, 2 * nn, s)) || (st = h2d(dB, B, 2 * nn, s)) || (st = h2d(dX, X, nn, s)) ||
      (st = h2d(dl, lambda, n, s)))
    return st;
  if ((st = ieig_stage1_dispatch(n, dA, n, dB, n, dX, n, dC, dBX, dM, form, slices, s))) return st;
  std::vector<double> M(nn);
  VCPCU_CUDA_TRY(cudaMemcpyAsync(M.data(), dM, nn * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  if (form != VCPCU_FORM_PLAIN && (st = take_status())) return st;
  if (inv(n, M.data(), ctx) != 0) {
    set_error("ieigsymge: the caller's inverse of mid(B X) failed");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = h2d(dM, M.data(), nn, s))) return st;
  if ((st = ieig_stage2_dispatch(n, dl, dM, n, dC, dBX, dlam, dG, form, slices, s))) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(lam, dlam, 2 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                                 s));
  VCPCU_CUDA_TRY(cudaMemcpyAsync(bound, dG, sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  if (form != VCPCU_FORM_PLAIN && (st = take_status())) return st;
  if (*bound >= 1.0) {
    set_error("ieigsymge: ||Y B X - I|| <= %.17g is not below 1", *bound);
    return VCPCU_ERR_VERIFY;
  }
  eig_merge_host(n, lam);
  return VCPCU_OK;
}

int vcpcu_ddgemm_dev(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                     double* C, int ldc, double* Cerr, int lde, int slices, void* stream) {
  clear_error();
  if (slices != 0 && (slices < 7 || slices > 14)) {
    set_error("ddgemm: slices must be 0 or in [7, 14], got %d", slices);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && (!A || !B)) || ldc < m || (k > 0 && (lda < m || ldb < k)) ||
      (Cerr && lde < m)) {
    set_error("ddgemm: null pointer or leading dimension too small");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (k > 0 && (misaligned16(A) || misaligned16(B))) {
    set_error("ddgemm: A and B must be 16-byte aligned (dd entries are read as pairs)");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  return ozaki_ddgemm(m, n, k, A, lda, B, ldb, C, ldc, Cerr, lde, slices, (cudaStream_t)stream);
}

int vcpcu_ddgemm(int m, int n, int k, const double* A, const double* B, double* C, double* Cerr,
                 int slices) {
  clear_error();
  if (slices != 0 && (slices < 7 || slices > 14)) {
    set_error("ddgemm: slices must be 0 or in [7, 14], got %d", slices);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && (!A || !B))) {
    set_error("ddgemm: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  cudaStream_t s = host_stream();
  const size_t na = 2 * (size_t)m * k, nb = 2 * (size_t)k * n, nc = 2 * (size_t)m * n,
               ne = Cerr ? (size_t)m * n : 0;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * (na + nb + nc + ne), s))) return st;
  double* dA = (double*)buf.ptr;
  double* dB = dA + na;
  double* dC = dB + nb;
  double* dE = Cerr ? dC + nc : nullptr;
  if ((st = h2d(dA, A, na, s)) || (st = h2d(dB, B, nb, s))) return st;
  if ((st = ozaki_ddgemm(m, n, k, dA, m, dB, k > 0 ? k : 1, dC, m, dE, m, slices, s))) return st;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(C, dC, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (Cerr)
    VCPCU_CUDA_TRY(cudaMemcpyAsync(Cerr, dE, ne * sizeof(double), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return take_status();
}

}  // extern "C"
