// common.cuh -- shared host/device helpers of libvcpcuda (status, errors,
// stream-ordered scratch, launch accounting).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cstdio>
#include <string>
#include <atomic>

#include "../../include/vcpcuda.h"

namespace vcpcu {

// ---- error reporting (thread-local text, read by vcpcu_last_error_string) ---
void set_error(const char* fmt, ...);
void clear_error();

// Record a launch of one of this library's kernels.
void count_launch(long long n = 1);

// Turn a CUDA error into VCPCU_ERR_CUDA with a message.
int cuda_fail(cudaError_t e, const char* what);

#define VCPCU_CUDA_TRY(expr)                                         \
  do {                                                               \
    cudaError_t _e = (expr);                                         \
    if (_e != cudaSuccess) return ::vcpcu::cuda_fail(_e, #expr);     \
  } while (0)

#define VCPCU_LAUNCH_CHECK(what)                                     \
  do {                                                               \
    cudaError_t _e = cudaGetLastError();                             \
    if (_e != cudaSuccess) return ::vcpcu::cuda_fail(_e, what);      \
    ::vcpcu::count_launch();                                         \
  } while (0)

// The device must be an sm_103 part (the only code this library carries).
int check_device();

// Stream-ordered scratch: a buffer from the current device's default memory
// pool (cudaMallocAsync), freed stream-ordered when the guard goes away.
struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  Scratch() = default;
  Scratch(const Scratch&) = delete;
  Scratch& operator=(const Scratch&) = delete;
  int alloc(size_t nbytes, cudaStream_t s);
  ~Scratch();
};

inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace vcpcu
