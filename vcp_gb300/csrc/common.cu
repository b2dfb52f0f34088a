// common.cu -- status/error plumbing and stream-ordered scratch.
#include "common.cuh"

#include <cstdarg>
#include <mutex>

namespace vcpcu {

static thread_local char g_err[1024] = {0};
static std::atomic<long long> g_launches{0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = 0; }

void count_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int cuda_fail(cudaError_t e, const char* what) {
  set_error("CUDA error in %s: %s (%d)", what, cudaGetErrorString(e), (int)e);
  return VCPCU_ERR_CUDA;
}

int check_device() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("no CUDA device: %s", cudaGetErrorString(e));
    return VCPCU_ERR_UNSUPPORTED;
  }
  // Cache the answer per device (up to 64 devices).
  static std::atomic<int> ok[64];
  if (dev < 64 && ok[dev].load() == 1) return VCPCU_OK;
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3) {
    set_error("libvcpcuda carries sm_103a code only; device %d is sm_%d%d", dev, major, minor);
    return VCPCU_ERR_UNSUPPORTED;
  }
  if (dev < 64) {
    // Keep freed pool memory cached: repeated calls then allocate for free.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    ok[dev].store(1);
  }
  return VCPCU_OK;
}

int Scratch::alloc(size_t nbytes, cudaStream_t s) {
  stream = s;
  bytes = nbytes;
  if (nbytes == 0) return VCPCU_OK;
  cudaError_t e = cudaMallocAsync(&ptr, nbytes, s);
  if (e != cudaSuccess) {
    ptr = nullptr;
    set_error("cudaMallocAsync(%zu bytes) failed: %s", nbytes, cudaGetErrorString(e));
    cudaGetLastError();
    return VCPCU_ERR_ALLOC;
  }
  return VCPCU_OK;
}

Scratch::~Scratch() {
  if (ptr) cudaFreeAsync(ptr, stream);
}

}  // namespace vcpcu

extern "C" {

const char* vcpcu_last_error_string(void) { return vcpcu::g_err; }

int vcpcu_version(void) { return 100; }

long long vcpcu_launch_count(void) { return vcpcu::g_launches.load(); }

}
