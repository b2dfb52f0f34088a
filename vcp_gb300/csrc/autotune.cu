// autotune.cu -- choice between the plain and the tensor-core form.
//
// VCPCU_FORM_AUTO runs the form with the smaller predicted time:
//   plain  t = 8 m n k / fp64_rate + t_launch
//   Ozaki  t = (L + 8) 2 Mp Np Kp / tc_rate            (slice GEMMs; L moduli)
//            + 16 (m k + k n) / prep_bw + 12 t_launch    (operand preparation)
// with the constants measured on this device by vcpcu_autotune (timing one
// plain and two Ozaki products), kept for the process and optionally stored
// in / loaded from the file named by VCPCU_AUTOTUNE_CACHE.  Until a
// calibration runs, conservative GB300 defaults are used.
#include "common.cuh"
#include "ozaki.cuh"
#include "variants.cuh"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <mutex>

namespace vcpcu {

namespace {

struct Model {
  double fp64_rate = 1.1e12;  // plain interval kernel, FP64 flops / s
  double tc_rate = 1.0e15;    // slice GEMM, bf16 flops / s
  double prep_bw = 1.5e12;    // bytes / s of the preparation kernels
  double t_launch = 5e-6;     // s per kernel launch
  bool calibrated = false;
};

Model g_model;
std::mutex g_model_mu;
bool g_loaded = false;

void load_cache_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const char* path = std::getenv("VCPCU_AUTOTUNE_CACHE");
  if (!path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  Model m;
  if (std::fscanf(f, "%lf %lf %lf %lf", &m.fp64_rate, &m.tc_rate, &m.prep_bw, &m.t_launch) == 4 &&
      m.fp64_rate > 0 && m.tc_rate > 0 && m.prep_bw > 0 && m.t_launch >= 0) {
    m.calibrated = true;
    g_model = m;
  }
  std::fclose(f);
}

double time_call(int m, int n, int k, int form, const double* A, const double* B, double* C,
                 cudaStream_t s, int reps) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  igemm_any(m, n, k, A, m, B, k, C, m, form, 0, s);  // warm-up
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps; ++r) igemm_any(m, n, k, A, m, B, k, C, m, form, 0, s);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms * 1e-3 / reps;
}

__global__ void fill_intervals(long n, double* X, unsigned seed) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)(i * 2654435761u) ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    const double mid = ((double)(h & 0xffffff) / 16777216.0) * 2.0 - 1.0;
    X[2 * i] = mid - 1e-12 * fabs(mid);
    X[2 * i + 1] = mid + 1e-12 * fabs(mid);
  }
}

}  // namespace

// Predicted seconds of a product in each form (for the AUTO choice).  In a
// batch (grouped launches) the per-product launch costs of both forms vanish.
int autotune_choose(int m, int n, int k, bool batched) {
  std::lock_guard<std::mutex> lk(g_model_mu);
  load_cache_locked();
  const Model& md = g_model;
  const double mnk = (double)m * n * (k > 0 ? k : 0);
  const double tl = batched ? 0.0 : md.t_launch;
  const double tp = 8.0 * mnk / md.fp64_rate + tl;
  const double Mp = std::ceil(m / 128.0) * 128.0, Np = std::ceil(n / 256.0) * 256.0,
               Kp = std::ceil((k > 0 ? k : 1) / 64.0) * 64.0;
  OzPlan plan;
  oz_make_plan(m, n, k, 8, 2, &plan, 1);
  const double gemms = plan.pb.L + 8.0;
  const double to = gemms * 2.0 * Mp * Np * Kp / md.tc_rate +
                    16.0 * ((double)m * k + (double)k * n) / md.prep_bw + 12.0 * tl;
  return to < tp ? VCPCU_FORM_OZAKI : VCPCU_FORM_PLAIN;
}

}  // namespace vcpcu

using namespace vcpcu;

extern "C" int vcpcu_autotune(void* stream, double* constants) {
  clear_error();
  int st = check_device();
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int n1 = 512, n2 = 1024, n3 = 2048;
  const size_t elems = 2 * (size_t)n3 * n3;
  Scratch buf;
  if ((st = buf.alloc(sizeof(double) * 3 * elems, s))) return st;
  double* A = (double*)buf.ptr;
  double* B = A + elems;
  double* C = B + elems;
  fill_intervals<<<1024, 256, 0, s>>>((long)n3 * n3, A, 1u);
  fill_intervals<<<1024, 256, 0, s>>>((long)n3 * n3, B, 2u);
  count_launch(2);
  const double tp = time_call(n1, n1, n1, VCPCU_FORM_PLAIN, A, B, C, s, 2);
  const double t2 = time_call(n2, n2, n2, VCPCU_FORM_OZAKI, A, B, C, s, 3);
  const double t3 = time_call(n3, n3, n3, VCPCU_FORM_OZAKI, A, B, C, s, 3);
  Model m;
  m.fp64_rate = 8.0 * n1 * (double)n1 * n1 / tp;
  // Ozaki: t = a * work + b, work = (L + 8) 2 n^3 (K multiple of the tiles here)
  OzPlan p2, p3;
  oz_make_plan(n2, n2, n2, 8, 2, &p2, 1);
  oz_make_plan(n3, n3, n3, 8, 2, &p3, 1);
  const double w2 = (p2.pb.L + 8.0) * 2.0 * n2 * (double)n2 * n2;
  const double w3 = (p3.pb.L + 8.0) * 2.0 * n3 * (double)n3 * n3;
  double a = (t3 - t2) / (w3 - w2);
  if (!(a > 0)) a = t3 / w3;
  double b = t2 - a * w2;
  if (b < 0) b = 0;
  m.tc_rate = 1.0 / a;
  // fixed cost b ~ preparation of 2 n2^2 entries + 12 launches
  m.t_launch = 5e-6;
  const double prep_t = b - 12.0 * m.t_launch;
  m.prep_bw = prep_t > 0 ? 16.0 * 2.0 * n2 * (double)n2 / prep_t : 5e12;
  m.calibrated = true;
  {
    std::lock_guard<std::mutex> lk(g_model_mu);
    g_model = m;
    g_loaded = true;
    const char* path = std::getenv("VCPCU_AUTOTUNE_CACHE");
    if (path) {
      FILE* f = std::fopen(path, "w");
      if (f) {
        std::fprintf(f, "%.17g %.17g %.17g %.17g\n", m.fp64_rate, m.tc_rate, m.prep_bw, m.t_launch);
        std::fclose(f);
      }
    }
  }
  if (constants) {
    constants[0] = m.fp64_rate;
    constants[1] = m.tc_rate;
    constants[2] = m.prep_bw;
    constants[3] = m.t_launch;
  }
  return VCPCU_OK;
}

extern "C" int vcpcu_autotune_choice(int m, int n, int k, int batched) {
  return autotune_choose(m, n, k, batched != 0);
}
