// noalloc.cu -- the Ozaki-form interval product for callers that cannot
// allocate device memory.
//
// Who needs it: code that runs where cudaMalloc / cudaMallocAsync are not
// allowed or not safe -- a real-time loop that must not hit the allocator
// (cudaMalloc can synchronise the device and its latency is unbounded), a
// process whose device memory is already owned by another allocator (a
// framework's caching pool, which would see its budget overrun), or an FFI
// caller whose contract is "no allocation after initialisation".  This entry point runs the same kernels as
// vcpcu_igemm_dev with form VCPCU_FORM_OZAKI, but takes its scratch from one
// file-scope static device array instead of the stream-ordered allocator.
//
// The array (VCPCU_NOALLOC_SCRATCH_BYTES, 32 MiB) exists on every device
// that loads this library, for the life of the process.  Every call shares
// it and it keeps the previous call's contents; each call re-initialises
// every word that must start at zero (the row maxima, digit and integer sums
// and status words are cleared on the call's stream; the digit and residue
// planes, fold buffer and radius bounds are fully overwritten).  Calls whose GPU work overlaps -- on
// two streams, or from two host threads without ordering -- race on the
// array and give wrong results: order them on one stream.
#include "common.cuh"
#include "ozaki.cuh"

#include <mutex>

namespace vcpcu {

namespace {

// The scratch of every no-allocation call on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[VCPCU_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device (host code cannot use the
// symbol itself: on the host it names a stand-in, not device memory).
void* g_scratch_ptr[64] = {nullptr};
std::mutex g_scratch_mu;

int scratch_for_current_device(void** out) {
  int dev = 0;
  VCPCU_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("igemm_noalloc: device ordinal %d out of range", dev);
    return VCPCU_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      set_error("igemm_noalloc: cudaGetSymbolAddress of the static scratch failed: %s",
                cudaGetErrorString(e));
      return VCPCU_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return VCPCU_OK;
}

}  // namespace

}  // namespace vcpcu

using namespace vcpcu;

extern "C" int vcpcu_igemm_noalloc_dev(int m, int n, int k, const double* A, int lda,
                                       const double* B, int ldb, double* C, int ldc,
                                       int slices, void* stream) {
  clear_error();
  const int sc = oz_slice_count(slices);
  if (sc != 0 && (sc < 2 || sc > OZ_MAX_SLICES)) {
    set_error("igemm_noalloc: slices must be 0 or in [2, %d] (optionally + "
              "VCPCU_SLICES_FAST_RADIUS), got %d", OZ_MAX_SLICES, slices);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (!C || (k > 0 && (!A || !B))) {
    set_error("igemm_noalloc: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (ldc < m || (k > 0 && (lda < m || ldb < k))) {
    set_error("igemm_noalloc: leading dimension too small (lda %d, ldb %d, ldc %d)", lda, ldb,
              ldc);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (k > 0 && (((uintptr_t)A | (uintptr_t)B) & 15) != 0) {
    set_error("igemm_noalloc: A and B must be 16-byte aligned (intervals are read as pairs)");
    return VCPCU_ERR_INVALID_ARG;
  }
  OzPlan plan;
  oz_make_plan(m, n, k, slices, 2, &plan, /*crt=*/1);
  const size_t need = oz_workspace_bytes(plan.pb);
  if (need > (size_t)VCPCU_NOALLOC_SCRATCH_BYTES) {
    set_error("igemm_noalloc: %d x %d x %d with %d slices needs %zu bytes of scratch, more than "
              "the %u-byte static scratch; use vcpcu_igemm_dev",
              m, n, k, plan.pb.s, need, (unsigned)VCPCU_NOALLOC_SCRATCH_BYTES);
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  void* base = nullptr;
  if ((st = scratch_for_current_device(&base))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  OzWorkspace ws;
  oz_carve_workspace(plan.pb, base, &ws);
  if ((st = oz_run_product(plan, ws, A, lda, B, ldb, C, ldc, s))) return st;
  // The reassembly already writes NaN everywhere after a non-finite input or
  // a timed-out wait; the status words go into the per-device status that
  // vcpcu_status reports, as for vcpcu_igemm_dev.
  oz_merge_status(ws.flag, s);
  VCPCU_LAUNCH_CHECK("oz_status_merge");
  return VCPCU_OK;
}
