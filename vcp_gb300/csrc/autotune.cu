// autotune.cu -- choice between the plain and the tensor-core form.
//
// VCPCU_FORM_AUTO runs the form with the smaller predicted time:
//   plain  t = 8 m n k / fp64_rate + t_launch
//   Ozaki  t = (L + 6) 2 Mp Np Kp / tc_rate            (slice GEMMs; L moduli,
//                                                       2 x 3 radius digit pairs)
//            + 16 (m k + k n) / prep_bw + 12 t_launch    (operand preparation)
// with the constants measured on this device by vcpcu_autotune (timing one
// plain and two Ozaki products), kept for the process and optionally stored
// in / loaded from the file named by VCPCU_AUTOTUNE_CACHE.  Until a
// calibration runs, conservative GB300 defaults are used.
//
// When the tensor-core form is the faster one, autotune_pick also chooses
// its slice count from the operands: the smallest s in {6, 7, 8, 9}
// (w = 42, 49, 56, 62 bit midpoints) with the fast radius products
// (VCPCU_SLICES_FAST_RADIUS: two bf16 GEMMs fewer) whose enclosures are no
// wider than the plain form's, then s = 8, 9 with the exact radius products
// (for radius factors whose magnitudes spread over many binades), else the
// plain form itself.  The choice is made per key
// (ceil log2 k, exponent spread of the rows of A plus the columns of B in
// steps of 4, radius-to-midpoint exponent in steps of 4), on a probe: a
// block of up to 64 rows of A and up to 64 evenly spaced columns of B,
// multiplied in the plain form and at every candidate s, the width ratios
// compared on the host; the result is kept for the process.
#include "common.cuh"
#include "ozaki.cuh"
#include "variants.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

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

// Exponent statistics of a sample: out[0] = max over the rows of the
// S_r x K block As (kv, ld S_r) of (largest - smallest exponent of a
// non-zero midpoint), out[1] the same over the columns of the K x S_c block
// Bs (ld K), out[2] = max over both of (exponent of the radius - exponent
// of the midpoint) where both are non-zero (INT_MIN + 1 if none).  One warp
// per row / column; midpoint and radius are (lo + up) / 2 and (up - lo) / 2
// in round-to-nearest (statistics only).
__device__ __forceinline__ void mid_rad_exp(const double* p, int* em, int* er) {
  const double lo = p[0], up = p[1];
  const double m = 0.5 * lo + 0.5 * up, r = 0.5 * up - 0.5 * lo;
  *em = m != 0.0 ? ilogb(m) : INT_MIN;
  *er = r > 0.0 ? ilogb(r) : INT_MIN;
}

__global__ void spread_stats_kernel(int Sr, int K, const double* __restrict__ As, int Sc,
                                    const double* __restrict__ Bs, int* __restrict__ out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= Sr + Sc) return;
  const bool row = warp < Sr;
  const int idx = row ? warp : warp - Sr;
  int emax = INT_MIN, emin = INT_MAX, rr = INT_MIN + 1;
  for (int p = lane; p < K; p += 32) {
    const double* e = row ? As + 2 * ((long)idx + (long)p * Sr) : Bs + 2 * ((long)p + (long)idx * K);
    int em, er;
    mid_rad_exp(e, &em, &er);
    if (em != INT_MIN) {
      emax = max(emax, em);
      emin = min(emin, em);
      if (er != INT_MIN) rr = max(rr, er - em);
    }
  }
  for (int o = 16; o; o >>= 1) {
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    emin = min(emin, __shfl_xor_sync(0xffffffffu, emin, o));
    rr = max(rr, __shfl_xor_sync(0xffffffffu, rr, o));
  }
  if (lane == 0) {
    if (emax != INT_MIN) atomicMax(out + (row ? 0 : 1), emax - emin);
    atomicMax(out + 2, rr);
  }
}

struct TuneKey {
  int klog, phi, rr;
  bool operator<(const TuneKey& o) const {
    return std::tie(klog, phi, rr) < std::tie(o.klog, o.phi, o.rr);
  }
};
std::map<TuneKey, int> g_slices;  // key -> slice count, 0 = plain form
std::mutex g_slices_mu;

// Accept slice count s on the probe's width ratios r (tensor-core / plain):
// the largest ratio must stay below 1 by at least 2^-16 and by a fifth of
// its distance from the 90th percentile (entries of the full product lie
// further out in the same tail), and when the ratios spread widely (largest
// above 4 x the median: large exponent spreads, whose tails are long) the
// largest must be at most 1/2.  Calibrated on the host models over inner
// dimensions 512 - 8192, exponent spreads 0 - 32 and radius ratios 0 -
// 2^-20: no accepted choice gave a wider entry of a 256 x 256 product.
bool probe_accepts(std::vector<double>& r) {
  if (r.empty()) return true;
  for (double v : r)
    if (!(v == v) || v == INFINITY) return false;
  std::sort(r.begin(), r.end());
  const size_t n = r.size();
  const double mx = r[n - 1], med = r[n / 2], q90 = r[(9 * n) / 10];
  const double gap = 1.0 - mx;
  if (gap < 0x1p-16 || gap < 0.2 * (mx - q90)) return false;
  if (mx > 4.0 * med && mx > 0.5) return false;
  return true;
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
  const double gemms = plan.pb.L + 2.0 * plan.rad.npairs;
  const double to = gemms * 2.0 * Mp * Np * Kp / md.tc_rate +
                    16.0 * ((double)m * k + (double)k * n) / md.prep_bw + 12.0 * tl;
  return to < tp ? VCPCU_FORM_OZAKI : VCPCU_FORM_PLAIN;
}

int autotune_pick(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                  cudaStream_t s, int* form, int* slices) {
  *form = autotune_choose(m, n, k);
  *slices = 0;
  if (*form == VCPCU_FORM_PLAIN || m <= 0 || n <= 0 || k <= 0) return VCPCU_OK;
  const int Sr = m < 64 ? m : 64, Sc = n < 64 ? n : 64;
  const int i0 = (m - Sr) / 2, cstride = n / Sc;
  // candidates in order of cost: s = 6, 7, 8, 9 with the fast radius
  // products, then 8 and 9 with the exact ones
  constexpr int NCAND = 6;
  const int cand[NCAND] = {6 | OZ_FAST_RADIUS, 7 | OZ_FAST_RADIUS, 8 | OZ_FAST_RADIUS,
                           9 | OZ_FAST_RADIUS, 8, 9};
  const size_t na = 2 * (size_t)Sr * k, nb = 2 * (size_t)k * Sc, nc = 2 * (size_t)Sr * Sc;
  Scratch buf;
  int st = buf.alloc(sizeof(double) * (na + nb + (NCAND + 1) * nc) + 64, s);
  if (st) return st;
  double* As = (double*)buf.ptr;
  double* Bs = As + na;
  double* Cs = Bs + nb;  // plain, then the candidates
  int* stats = (int*)(Cs + (NCAND + 1) * nc);
  VCPCU_CUDA_TRY(cudaMemcpy2DAsync(As, Sr * 16, A + 2 * (size_t)i0, lda * 16, Sr * 16, k,
                                   cudaMemcpyDefault, s));
  for (int c = 0; c < Sc; ++c)  // column c * cstride of B (contiguous)
    VCPCU_CUDA_TRY(cudaMemcpyAsync(Bs + 2 * (size_t)k * c, B + 2 * (size_t)c * cstride * ldb,
                                   (size_t)k * 16, cudaMemcpyDefault, s));
  const int init[3] = {0, 0, INT_MIN + 1};
  VCPCU_CUDA_TRY(cudaMemcpyAsync(stats, init, sizeof(init), cudaMemcpyHostToDevice, s));
  spread_stats_kernel<<<(Sr + Sc + 7) / 8, 256, 0, s>>>(Sr, k, As, Sc, Bs, stats);
  VCPCU_LAUNCH_CHECK("spread_stats_kernel");
  int h[3];
  VCPCU_CUDA_TRY(cudaMemcpyAsync(h, stats, sizeof(h), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  int klog = 0;
  while ((1L << klog) < k) ++klog;
  const int phi = (h[0] + h[1] + 3) / 4;
  const int rr = h[2] <= -80 ? -1000 : (h[2] >= 0 ? 0 : -((-h[2]) / 4));
  const TuneKey key{klog, phi, rr};
  {
    std::lock_guard<std::mutex> lk(g_slices_mu);
    auto it = g_slices.find(key);
    if (it != g_slices.end()) {
      *slices = it->second;
      *form = it->second ? VCPCU_FORM_OZAKI : VCPCU_FORM_PLAIN;
      return VCPCU_OK;
    }
  }
  // probe: the plain form and every candidate on the sampled block
  if ((st = igemm_any(Sr, Sc, k, As, Sr, Bs, k, Cs, Sr, VCPCU_FORM_PLAIN, 0, s))) return st;
  for (int c = 0; c < NCAND; ++c)
    if ((st = ozaki_igemm(Sr, Sc, k, As, Sr, Bs, k, Cs + (c + 1) * nc, Sr, VCPCU_FORM_OZAKI,
                          cand[c], s)))
      return st;
  std::vector<double> hc((NCAND + 1) * nc);
  VCPCU_CUDA_TRY(cudaMemcpyAsync(hc.data(), Cs, sizeof(double) * (NCAND + 1) * nc,
                                 cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  int choice = 0;
  for (int c = 0; c < NCAND && !choice; ++c) {
    std::vector<double> r;
    r.reserve(nc / 2);
    const double* P = hc.data();
    const double* O = hc.data() + (c + 1) * nc;
    for (size_t e = 0; e < nc / 2; ++e) {
      const double wp = P[2 * e + 1] - P[2 * e], wo = O[2 * e + 1] - O[2 * e];
      r.push_back(wp > 0.0 ? wo / wp : (wo > 0.0 ? INFINITY : 0.0));
    }
    if (probe_accepts(r)) choice = cand[c];
  }
  {
    std::lock_guard<std::mutex> lk(g_slices_mu);
    g_slices[key] = choice;
  }
  *slices = choice;
  *form = choice ? VCPCU_FORM_OZAKI : VCPCU_FORM_PLAIN;
  return VCPCU_OK;
}

}  // namespace vcpcu

using namespace vcpcu;

extern "C" int vcpcu_autotune_pick(int m, int n, int k, const double* A, int lda, const double* B,
                                   int ldb, int* form, int* slices, void* stream) {
  clear_error();
  if (!form || !slices) {
    set_error("autotune_pick: null output pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (m > 0 && n > 0 && k > 0 && (!A || !B || lda < m || ldb < k)) {
    set_error("autotune_pick: null operand or leading dimension too small");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  return autotune_pick(m, n, k, A, lda, B, ldb, (cudaStream_t)stream, form, slices);
}

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
  // Ozaki: t = a * work + b, work = (L + 6) 2 n^3 (K multiple of the tiles here)
  OzPlan p2, p3;
  oz_make_plan(n2, n2, n2, 8, 2, &p2, 1);
  oz_make_plan(n3, n3, n3, 8, 2, &p3, 1);
  const double w2 = (p2.pb.L + 2.0 * p2.rad.npairs) * 2.0 * n2 * (double)n2 * n2;
  const double w3 = (p3.pb.L + 2.0 * p3.rad.npairs) * 2.0 * n3 * (double)n3 * n3;
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
    std::lock_guard<std::mutex> lk(g_slices_mu);
    g_slices.clear();  // slice choices are re-made under the new constants
  }
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
