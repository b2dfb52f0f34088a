// ozaki.cu -- orchestration of the Ozaki-form interval product:
//   plan (slice counts, pair lists, fixed-point scaling), scratch layout,
//   operand preparation, the three slice-GEMM phases
//     1. T  = RU(P^ * rB^)        P = |mA| +ru rA, both factors rounded up
//     2. T += RU(rA^ * |mB|^)
//     3. C  = [RD(mA mB) - e, RU(mA mB) + e], e = RU(truncation + T)
//   (one launch for the CRT form, whose phase 3 is the residue GEMMs and
//   the reassembly; three for the slices form)
// which together enclose pidblas's midpoint-radius product
// (vcp/pidblas.hpp:239-294): mA*mB from the truncated slice expansion plus
// its rigorous truncation bound, and the radius term
// (|mA| + rA) * rB + rA * |mB| bounded from above.
#include "common.cuh"
#include "ozaki.cuh"
#include "ozaki_common.cuh"
#include "tc_ptx.cuh"

#include <cmath>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

namespace vcpcu {

namespace {

void build_pairs(int sa, int sb, bool triangular, OzPairList* pl) {
  memset(pl, 0, sizeof(*pl));
  const int tmax = triangular ? (sa > sb ? sa : sb) + 1 : sa + sb;
  int n = 0, g = 0;
  for (int t = 2; t <= tmax; ++t) {
    const int start = n;
    for (int p = 1; p < t; ++p) {
      const int q = t - p;
      if (p > sa || q > sb) continue;
      pl->pa[n] = (int8_t)(p - 1);
      pl->pb[n] = (int8_t)(q - 1);
      pl->pt[n] = (int8_t)t;
      ++n;
    }
    if (n > start) {
      pl->gstart[g] = (int16_t)start;
      pl->gt[g] = (int8_t)t;
      ++g;
    }
  }
  pl->gstart[g] = (int16_t)n;
  pl->npairs = n;
  pl->ngroups = g;
}

// The radius products' pairs in one group (t ascending, p ascending), each
// pair weighted by 2^(8 (t_ref - t)) in the epilogue's fp32 upward sum; gt
// of the group is the largest t.  low_out (CRT form with OZ_FAST_RADIUS,
// sr = 2): the pairs with t <= 3 -- the pair of the two low digits is left
// out and bounded in the reassembly (sum_k lo_A lo_B <= sqrt(sum lo_A^2)
// sqrt(sum lo_B^2), weight 2^-8 against t_ref = 3): three tensor-core
// products per radius product instead of four.  Else all sr x sr pairs.
void radius_pairs(int sr, bool low_out, OzPairList* pl) {
  build_pairs(sr, sr, low_out, pl);
  pl->gt[0] = pl->gt[pl->ngroups - 1];
  pl->gstart[1] = (int16_t)pl->npairs;
  pl->ngroups = 1;
}

// Largest t_ref keeping |W| < 2^62, and the number of floored folds.
void choose_scaling(const OzPairList& pl, int nchunks, int* t_ref, int* R) {
  int best = 2;
  const int tmax = pl.gt[pl.ngroups - 1];
  for (int tr = 2; tr <= tmax; ++tr) {
    double bound = 0.0;
    for (int g = 0; g < pl.ngroups; ++g) {
      const double np = (double)(pl.gstart[g + 1] - pl.gstart[g]);
      bound += np * nchunks * 16777216.0 * std::ldexp(1.0, 8 * (tr - pl.gt[g])) + 64.0;
    }
    if (bound < std::ldexp(1.0, 62)) best = tr;
  }
  int r = 0;
  for (int g = 0; g < pl.ngroups; ++g) {
    if (pl.gt[g] <= best) continue;
    const int total = (pl.gstart[g + 1] - pl.gstart[g]) * nchunks;
    r += (total + OZ_FOLD_CHUNKS - 1) / OZ_FOLD_CHUNKS;
  }
  *t_ref = best;
  *R = r;
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// Sticky per-device status of the Ozaki form: bit 0 non-finite input, bit 1
// a bounded device wait timed out.  Merged after every product, read and
// cleared by oz_take_status.
__device__ int g_oz_status;

__global__ void oz_status_merge(const int* flag) {
  int v = (flag[0] ? 1 : 0) | (flag[1] ? 2 : 0);
  if (v) atomicOr(&g_oz_status, v);
}

// Optional per-phase timing (CUDA events recorded on the call's stream).
struct OzProfile {
  bool on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[5];  // prep, rad1, rad2, mid, reassembly
  long long flops = 0;
};
OzProfile g_prof;
std::mutex g_prof_mu;

}  // namespace

PhaseTimer::PhaseTimer(int ph, cudaStream_t st) : phase(ph), s(st) {
  if (!g_prof.on) return;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, s);
}

PhaseTimer::~PhaseTimer() {
  if (!a) return;
  cudaEventRecord(b, s);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.ev[phase].emplace_back(a, b);
}

void oz_profile_add_flops(long long f) {
  if (!g_prof.on) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.flops += f;
}

int oz_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.on = on != 0;
  return VCPCU_OK;
}

int oz_profile_read(double* ms, int nphases, long long* flops) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (int ph = 0; ph < 5; ++ph) {
    double tot = 0.0;
    for (auto& e : g_prof.ev[ph]) {
      cudaEventSynchronize(e.second);
      float t = 0.f;
      cudaEventElapsedTime(&t, e.first, e.second);
      tot += t;
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
    g_prof.ev[ph].clear();
    if (ph < nphases && ms) ms[ph] = tot;
  }
  if (flops) *flops = g_prof.flops;
  g_prof.flops = 0;
  return VCPCU_OK;
}

// Self-test of the timeout path: one thread waits, with the bounded wait of
// the slice GEMM (mbar_wait), on an mbarrier that nothing ever arrives on;
// the wait gives up after `limit` cycles and the kernel sets the timeout
// word (flag[1]) and returns -- no fault, trap or hang.
__global__ void oz_wait_selftest(int* flag, long long limit) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    ptx::mbar_init(&bar, 1);
    ptx::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !ptx::mbar_wait(&bar, 0, limit)) flag[1] = 1;
}

int oz_selftest_timeout(long long limit, cudaStream_t s) {
  Scratch fl;
  int st = fl.alloc(4 * sizeof(int), s);
  if (st) return st;
  VCPCU_CUDA_TRY(cudaMemsetAsync(fl.ptr, 0, 4 * sizeof(int), s));
  oz_wait_selftest<<<1, 32, 0, s>>>((int*)fl.ptr, limit);
  VCPCU_LAUNCH_CHECK("oz_wait_selftest");
  oz_merge_status((const int*)fl.ptr, s);
  return VCPCU_OK;
}

void oz_merge_status(const int* flag, cudaStream_t s) {
  oz_status_merge<<<1, 1, 0, s>>>(flag);
  count_launch();
}

int* oz_status_ptr() {
  static std::mutex mu;
  static int* ptr[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_oz_status) != cudaSuccess) return nullptr;
    ptr[dev] = (int*)p;
  }
  return ptr[dev];
}

int oz_take_status(cudaStream_t s, int* status) {
  int zero = 0;
  VCPCU_CUDA_TRY(cudaMemcpyFromSymbolAsync(status, g_oz_status, sizeof(int), 0,
                                           cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  VCPCU_CUDA_TRY(cudaMemcpyToSymbolAsync(g_oz_status, &zero, sizeof(int), 0,
                                         cudaMemcpyHostToDevice, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return VCPCU_OK;
}

// CRT form: number of moduli L and basis Q_l for w-bit operands and inner
// dimension K: the product A'B' satisfies |A'B'| <= K 2^(2w-2); the moduli
// are taken with prod m_l > K 2^(2w) = 4 max |A'B'|, so the centred value
// lies within a quarter of M of zero and the reassembly's quotient needs no
// correction step.
// Returns 0, or -1 if 16 moduli do not suffice.
int crt_setup(int K, int w, OzPlan* plan) {
  const double need = 2.0 * w + std::log2((double)(K > 1 ? K : 1)) + 0.01;
  double bits = 0.0;
  int L = 0;
  while (L < OZ_MAX_MODULI_128 && bits <= need) bits += std::log2((double)OZ_MODULI[L++]);
  if (bits <= need) return -1;
  unsigned __int128 Mv = 1;
  for (int l = 0; l < L; ++l) Mv *= (unsigned __int128)OZ_MODULI[l];
  for (int l = 0; l < L; ++l) {
    const int m = OZ_MODULI[l];
    const unsigned __int128 Ml = Mv / (unsigned __int128)m;
    const int r = (int)(Ml % (unsigned __int128)m);
    int inv = 0;
    for (int x = 1; x < m; ++x)
      if ((r * x) % m == 1) {
        inv = x;
        break;
      }
    const unsigned __int128 Q = Ml * (unsigned __int128)inv;  // < M
    for (int t = 0; t < 4; ++t) plan->Q[l][t] = (uint32_t)(Q >> (32 * t));
  }
  for (int t = 0; t < 4; ++t) plan->Mlimb[t] = (uint32_t)(Mv >> (32 * t));
  plan->pb.L = L;
  return 0;
}

static_assert(OZ_FAST_RADIUS == VCPCU_SLICES_FAST_RADIUS, "slices flag of the C ABI");

int oz_make_plan(int M, int N, int K, int s, int sr, OzPlan* plan, int crt) {
  memset(plan, 0, sizeof(*plan));
  const bool fast_rad = (s & OZ_FAST_RADIUS) != 0;
  s = oz_slice_count(s);
  if (s <= 0) s = 8;
  OzProblem& pb = plan->pb;
  pb.M = M;
  pb.N = N;
  pb.K = K;
  pb.Mp = (M + OZ_BM - 1) / OZ_BM * OZ_BM;
  pb.Np = (N + OZ_BN - 1) / OZ_BN * OZ_BN;
  pb.Kp = K <= 0 ? OZ_BK : (K + OZ_BK - 1) / OZ_BK * OZ_BK;
  pb.s = s;
  pb.sr = sr;
  build_pairs(s, s, true, &plan->mid);
  plan->rad_lowb = crt != 0 && fast_rad;
  radius_pairs(sr, plan->rad_lowb != 0, &plan->rad);
  pb.mplanes = s;
  if (crt) {
    pb.crt = 1;
    pb.w = 7 * s < 62 ? 7 * s : 62;  // |A'|, |B'| <= 2^61 stay 64-bit integers
    const int Keff = pb.K > 1 ? pb.K : 1;
    while (crt_setup(Keff, pb.w, plan) != 0) --pb.w;  // very long K: fewer bits per operand
    pb.mplanes = pb.L;
    OzPairList& pl = plan->crt;
    memset(&pl, 0, sizeof(pl));
    for (int l = 0; l < pb.L; ++l) {
      pl.pa[l] = (int8_t)l;
      pl.pb[l] = (int8_t)l;
      pl.gstart[l] = (int16_t)l;
      pl.gt[l] = (int8_t)l;
    }
    pl.gstart[pb.L] = (int16_t)pb.L;
    pl.npairs = pl.ngroups = pb.L;
  }
  const int nchunks = (pb.Kp + OZ_CHUNK - 1) / OZ_CHUNK;
  choose_scaling(plan->mid, nchunks, &plan->t_ref_mid, &plan->R_mid);
  choose_scaling(plan->rad, nchunks, &plan->t_ref_rad, &plan->R_rad);
  // one fold per radius product: the slice GEMM's fp32 upward sum of all
  // its digit pairs, already weighted by 2^(8 (t_ref - t))
  plan->rad_slots = 1;
  return VCPCU_OK;
}

OzRadConst oz_rad_const(const OzPlan& plan) {
  OzRadConst rc;
  memset(&rc, 0, sizeof(rc));
  rc.nslot = plan.rad_slots;
  rc.run1 = !(plan.point_mask & 2);
  rc.run2 = !(plan.point_mask & 1);
  rc.t_ref = plan.t_ref_rad;
  rc.R = plan.R_rad;
  rc.lowb = plan.rad_lowb;
  return rc;
}

namespace {
// folds per radius product of a problem (one: the epilogue's fp32 sum)
int rad_slot_count(const OzProblem&) { return 1; }
}  // namespace

size_t oz_workspace_bytes(const OzProblem& pb) {
  const size_t np = (size_t)(pb.mplanes + 2 * pb.sr);
  size_t b = 0;
  b += al256(np * pb.Mp * pb.Kp * 2);
  b += al256(np * pb.Np * pb.Kp * 2);
  b += al256(sizeof(unsigned long long) * 3 * pb.Mp);
  b += al256(sizeof(int) * 3 * pb.Mp);
  b += al256(sizeof(unsigned long long) * pb.Mp);
  b += al256(sizeof(int) * 2 * pb.Np);
  b += al256(sizeof(double) * pb.Np);
  if (!pb.crt) {  // T and the midpoint fold buffer: slice form only
    b += al256(sizeof(double) * (size_t)pb.Mp * pb.Np);
    b += al256(sizeof(long long) * (size_t)pb.Mp * pb.Np);
  }
  b += al256(sizeof(int32_t) * 2 * (size_t)rad_slot_count(pb) * pb.Mp * pb.Np);
  b += al256(sizeof(int) * 4);
  b += 2 * al256(sizeof(double) * (size_t)pb.M * (pb.K > 0 ? pb.K : 1));
  b += 2 * al256(sizeof(double) * (size_t)pb.Np * pb.Kp);
  if (pb.crt) b += al256(sizeof(unsigned long long) * 4 * pb.Np);
  b += al256(sizeof(unsigned long long) * 4 * pb.Mp);
  if (pb.crt) b += al256((size_t)pb.L * pb.Np * pb.Mp);
  return b;
}

int oz_carve_workspace(const OzProblem& pb, void* base, OzWorkspace* ws) {
  uint8_t* p = (uint8_t*)base;
  const size_t mk = (size_t)pb.Mp * pb.Kp, nk = (size_t)pb.Np * pb.Kp;
  const size_t np = (size_t)(pb.mplanes + 2 * pb.sr);
  uint16_t* a = (uint16_t*)p;
  ws->a_mid = a;
  ws->a_p = a + pb.mplanes * mk;
  ws->a_r = ws->a_p + pb.sr * mk;
  p += al256(np * mk * 2);
  uint16_t* b = (uint16_t*)p;
  ws->b_mid = b;
  ws->b_r = b + pb.mplanes * nk;
  ws->b_s = ws->b_r + pb.sr * nk;
  p += al256(np * nk * 2);
  ws->rowmax = (unsigned long long*)p;
  p += al256(sizeof(unsigned long long) * 3 * pb.Mp);
  ws->E3 = (int*)p;
  p += al256(sizeof(int) * 3 * pb.Mp);
  ws->delta = (unsigned long long*)p;
  p += al256(sizeof(unsigned long long) * pb.Mp);
  ws->F2 = (int*)p;
  p += al256(sizeof(int) * 2 * pb.Np);
  ws->beta = (double*)p;
  p += al256(sizeof(double) * pb.Np);
  ws->T = nullptr;
  ws->W = nullptr;
  if (!pb.crt) {
    ws->T = (double*)p;
    p += al256(sizeof(double) * (size_t)pb.Mp * pb.Np);
    ws->W = (long long*)p;
    p += al256(sizeof(long long) * (size_t)pb.Mp * pb.Np);
  }
  ws->P = (int32_t*)p;
  p += al256(sizeof(int32_t) * 2 * (size_t)rad_slot_count(pb) * pb.Mp * pb.Np);
  ws->flag = (int*)p;
  p += al256(sizeof(int) * 4);
  const size_t mk1 = sizeof(double) * (size_t)pb.M * (pb.K > 0 ? pb.K : 1);
  ws->midA = (double*)p;
  p += al256(mk1);
  ws->radA = (double*)p;
  p += al256(mk1);
  ws->midB = (double*)p;
  p += al256(sizeof(double) * (size_t)pb.Np * pb.Kp);
  ws->radB = (double*)p;
  p += al256(sizeof(double) * (size_t)pb.Np * pb.Kp);
  ws->bsum = nullptr;
  if (pb.crt) {
    ws->bsum = (unsigned long long*)p;
    p += al256(sizeof(unsigned long long) * 4 * pb.Np);
  }
  ws->asum = (unsigned long long*)p;
  p += al256(sizeof(unsigned long long) * 4 * pb.Mp);
  ws->res = pb.crt ? (uint8_t*)p : nullptr;
  return VCPCU_OK;
}

int oz_run_product(const OzPlan& plan, OzWorkspace& ws, const double* A, long lda,
                   const double* B, long ldb, double* C, long ldc, cudaStream_t s) {
  int st;
  {
    PhaseTimer t(0, s);
    if ((st = oz_prepare(plan.pb, A, lda, B, ldb, ws, s))) return st;
  }
  // T = (|mA| + rA) * rB + rA * |mB|: each product leaves its folds in its
  // half of ws.P.  A product with a zero factor would give exactly 0 (its
  // exponent is the zero sentinel), so it is skipped; the reassembly (CRT
  // form) or oz_radius_T (slice form) combines what ran.
  if (plan.pb.crt) {
    // CRT form: the radius products and the residue GEMMs in one launch
    // (phase 3 times all of them)
    PhaseTimer t(3, s);
    if ((st = oz_run_gemm(plan, OZ_ALL, ws, nullptr, 0, s))) return st;
  } else {
    if (!(plan.point_mask & 2)) {
      PhaseTimer t(1, s);
      if ((st = oz_run_gemm(plan, OZ_RAD_SET, ws, nullptr, 0, s))) return st;
    }
    if (!(plan.point_mask & 1)) {
      PhaseTimer t(2, s);
      if ((st = oz_run_gemm(plan, OZ_RAD_ADD, ws, nullptr, 0, s))) return st;
    }
    if ((st = oz_radius_T(plan, ws, s))) return st;
    PhaseTimer t(3, s);
    if ((st = oz_run_gemm(plan, OZ_MID, ws, C, ldc, s))) return st;
  }
  if (plan.pb.crt) {
    PhaseTimer t(4, s);
    if ((st = oz_crt_assemble(plan, ws, C, ldc, s))) return st;
  }
  return VCPCU_OK;
}

namespace {

__global__ void oz_fill_nan(size_t count, double* C) {
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (size_t)gridDim.x * blockDim.x)
    C[i] = nan;
}

// Events of one pipelined call, and the streams it must drain before its
// device memory goes back to the pool (also on error paths).
struct PipeGuard {
  std::vector<cudaEvent_t> ev;
  cudaStream_t streams[5];
  PipeGuard(cudaStream_t a, cudaStream_t b, cudaStream_t c, cudaStream_t d, cudaStream_t e)
      : streams{a, b, c, d, e} {}
  cudaEvent_t make() {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    ev.push_back(e);
    return e;
  }
  ~PipeGuard() {
    for (cudaStream_t x : streams) cudaStreamSynchronize(x);
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
};

int pipe_event(PipeGuard& g, cudaStream_t rec, cudaStream_t waiter) {
  cudaEvent_t e = g.make();
  if (!e) {
    set_error("cudaEventCreateWithFlags failed");
    cudaGetLastError();
    return VCPCU_ERR_CUDA;
  }
  VCPCU_CUDA_TRY(cudaEventRecord(e, rec));
  VCPCU_CUDA_TRY(cudaStreamWaitEvent(waiter, e, 0));
  return VCPCU_OK;
}

}  // namespace

namespace {
// Boundaries of about `parts` blocks over `len` entries, multiples of
// `unit` except the end; the first block is half the size of the others.
std::vector<int> block_bounds(int len, int parts, int unit) {
  std::vector<int> b{0};
  if (parts > 1) {
    for (int t = 1; t < parts; ++t) {
      const double x = (double)len * (t - 0.5) / (parts - 0.5);
      const int c = ((int)x + unit - 1) / unit * unit;
      if (c > b.back() && c < len) b.push_back(c);
    }
  }
  b.push_back(len);
  return b;
}
}  // namespace

int ozaki_igemm_host_pipelined(int m, int n, int k, const double* A, const double* B, double* C,
                               int slices, int panels, int row_panels, cudaStream_t s,
                               cudaStream_t c0, cudaStream_t c1, cudaStream_t up,
                               cudaStream_t down) {
  const int nslices = slices > 0 ? slices : 8;
  if (k > (1 << 20)) {
    set_error("igemm (Ozaki form): inner dimension %d above the supported 2^20", k);
    return VCPCU_ERR_UNSUPPORTED;
  }
  if (m <= 0 || n <= 0) return VCPCU_OK;
  if (k < 0) k = 0;
  if (panels < 1) panels = 1;
  if (row_panels < 1) row_panels = 1;
  OzPlan plan;  // the whole product: its workspace holds every block's planes
  oz_make_plan(m, n, k, nslices, 2, &plan, 1);
  const OzProblem& pb = plan.pb;
  // block boundaries (whole row / column tiles); the first blocks, waited
  // for before anything computes, are half the size of the others
  const std::vector<int> rb = block_bounds(m, row_panels, OZ_BM),
                         cb = block_bounds(n, panels, OZ_BN);
  row_panels = (int)rb.size() - 1;
  panels = (int)cb.size() - 1;
  // residue bytes and radius folds of one block product (as laid out by
  // oz_carve_workspace for its plan): the whole product's buffers serve the
  // products on c0, a second pair sized for the largest block those on c1
  auto blk_res = [&](int mv, int wj) {
    const size_t Mp = (size_t)(mv + OZ_BM - 1) / OZ_BM * OZ_BM,
                 Np = (size_t)(wj + OZ_BN - 1) / OZ_BN * OZ_BN;
    return al256((size_t)pb.L * Np * Mp);
  };
  auto blk_P = [&](int mv, int wj) {
    const size_t Mp = (size_t)(mv + OZ_BM - 1) / OZ_BM * OZ_BM,
                 Np = (size_t)(wj + OZ_BN - 1) / OZ_BN * OZ_BN;
    return al256(sizeof(int32_t) * 2 * (size_t)plan.rad_slots * Mp * Np);
  };
  size_t res1 = 0, P1 = 0;  // the largest block of each shape the loop below makes
  for (int t = 0; t < row_panels || t < panels; ++t) {
    const int nj = t < panels ? t : panels, ni = t + 1 < row_panels ? t + 1 : row_panels;
    if (t < row_panels)
      for (int J = 0; J < nj; ++J) {  // row block t against columns [0, nj) or one block
        res1 = std::max(res1, blk_res(rb[t + 1] - rb[t], cb[nj] - cb[0]));
        P1 = std::max(P1, blk_P(rb[t + 1] - rb[t], cb[nj] - cb[0]));
      }
    if (t < panels) {
      res1 = std::max(res1, blk_res(rb[ni] - rb[0], cb[t + 1] - cb[t]));
      P1 = std::max(P1, blk_P(rb[ni] - rb[0], cb[t + 1] - cb[t]));
    }
  }
  const size_t na = 2 * (size_t)m * k, nbe = 2 * (size_t)k * n, nc = 2 * (size_t)m * n;
  const size_t off_b = al256(na * 8), off_c = off_b + al256(nbe * 8),
               off_w = off_c + al256(nc * 8), off_r1 = off_w + al256(oz_workspace_bytes(pb)),
               off_p1 = off_r1 + res1;
  Scratch buf;
  int st = buf.alloc(off_p1 + P1, s);
  if (st) return st;
  PipeGuard g(s, c0, c1, up, down);  // destroyed before buf: drains every stream first
  double* dA = (double*)buf.ptr;
  double* dB = (double*)((uint8_t*)buf.ptr + off_b);
  double* dC = (double*)((uint8_t*)buf.ptr + off_c);
  OzWorkspace ws;
  oz_carve_workspace(pb, (uint8_t*)buf.ptr + off_w, &ws);
  uint8_t* res1p = (uint8_t*)buf.ptr + off_r1;
  int32_t* P1p = (int32_t*)((uint8_t*)buf.ptr + off_p1);
  // the other streams may touch the memory only after its allocation on s
  if ((st = pipe_event(g, s, up)) || (st = pipe_event(g, s, down)) ||
      (st = pipe_event(g, s, c0)) || (st = pipe_event(g, s, c1)))
    return st;
  if ((st = oz_prepare_left_begin(pb, ws, s))) return st;

  // uploads, interleaved: A's row block t, then B's column block t
  const size_t rowb = 2 * sizeof(double);  // bytes of one interval
  std::vector<cudaEvent_t> evA(row_panels), evB(panels);
  for (int t = 0; t < row_panels || t < panels; ++t) {
    if (t < row_panels) {
      const int i0 = rb[t], mv = rb[t + 1] - rb[t];
      if (k > 0)
        VCPCU_CUDA_TRY(cudaMemcpy2DAsync(dA + 2 * (size_t)i0, m * rowb, A + 2 * (size_t)i0,
                                         m * rowb, mv * rowb, k, cudaMemcpyHostToDevice, up));
      if (!(evA[t] = g.make())) return cuda_fail(cudaErrorUnknown, "cudaEventCreate");
      VCPCU_CUDA_TRY(cudaEventRecord(evA[t], up));
    }
    if (t < panels) {
      const int j0 = cb[t], wj = cb[t + 1] - cb[t];
      if (k > 0)
        VCPCU_CUDA_TRY(cudaMemcpyAsync(dB + 2 * (size_t)j0 * k, B + 2 * (size_t)j0 * k,
                                       2 * (size_t)wj * k * sizeof(double),
                                       cudaMemcpyHostToDevice, up));
      if (!(evB[t] = g.make())) return cuda_fail(cudaErrorUnknown, "cudaEventCreate");
      VCPCU_CUDA_TRY(cudaEventRecord(evB[t], up));
    }
  }

  // the part of C over row blocks [I0, I1) and column blocks [J0, J1): its
  // slice GEMMs on views of the whole planes, its reassembly, its download;
  // products alternate between c0 and c1, each after the preparations
  // issued on s so far (those of its operand blocks)
  long long flops = 0;
  int nblk = 0;
  auto block = [&](int I0, int I1, int J0, int J1) -> int {
    const int i0 = rb[I0], mv = rb[I1] - rb[I0];
    const int j0 = cb[J0], wj = cb[J1] - cb[J0];
    if (mv <= 0 || wj <= 0) return VCPCU_OK;
    OzPlan pj;
    oz_make_plan(mv, wj, k, nslices, 2, &pj, 1);
    OzWorkspace v = ws;
    const size_t Kp = (size_t)pb.Kp;
    v.a_mid = ws.a_mid + (size_t)i0 * Kp;
    v.a_p = ws.a_p + (size_t)i0 * Kp;
    v.a_r = ws.a_r + (size_t)i0 * Kp;
    v.a_pstride = (size_t)pb.Mp * Kp;
    v.b_mid = ws.b_mid + (size_t)j0 * Kp;
    v.b_r = ws.b_r + (size_t)j0 * Kp;
    v.b_s = ws.b_s + (size_t)j0 * Kp;
    v.b_pstride = (size_t)pb.Np * Kp;
    v.rowmax = ws.rowmax + 3 * (size_t)i0;
    v.E3 = ws.E3 + 3 * (size_t)i0;
    v.delta = ws.delta + i0;
    v.asum = ws.asum + 4 * (size_t)i0;
    v.F2 = ws.F2 + 2 * (size_t)j0;
    v.beta = ws.beta + j0;
    v.bsum = ws.bsum + 4 * (size_t)j0;
    const bool odd = (nblk++ & 1) != 0;
    cudaStream_t c = odd ? c1 : c0;
    if (odd) {
      v.res = res1p;
      v.P = P1p;
    }
    int e;
    if ((e = pipe_event(g, s, c))) return e;
    if ((e = oz_run_gemm(pj, OZ_ALL, v, nullptr, 0, c))) return e;
    double* cblk = dC + 2 * ((size_t)i0 + (size_t)j0 * m);
    if ((e = oz_crt_assemble(pj, v, cblk, m, c))) return e;
    if ((e = pipe_event(g, c, down))) return e;
    VCPCU_CUDA_TRY(cudaMemcpy2DAsync(C + 2 * ((size_t)i0 + (size_t)j0 * m), m * rowb, cblk,
                                     m * rowb, mv * rowb, wj, cudaMemcpyDeviceToHost, down));
    flops += 2LL * mv * wj * (long long)k * (pj.pb.L + 2LL * pj.rad.npairs);
    return VCPCU_OK;
  };
  // compute in arrival order: each new row block of A meets the column
  // blocks of B already prepared (one product over their contiguous
  // columns), each new column block the row blocks (one product over their
  // rows); after the last upload, block by block, so that the download of
  // one overlaps the next
  const bool last_is_b = panels >= row_panels;
  for (int t = 0; t < row_panels || t < panels; ++t) {
    if (t < row_panels) {
      const int i0 = rb[t], rows = (t + 1 < row_panels ? rb[t + 1] : pb.Mp) - i0;
      VCPCU_CUDA_TRY(cudaStreamWaitEvent(s, evA[t], 0));
      if ((st = oz_prepare_left_rows(pb, dA, m, i0, rows, ws, s))) return st;
      const int nj = t < panels ? t : panels;
      if (!last_is_b && t == row_panels - 1) {
        for (int J = 0; J < nj; ++J)
          if ((st = block(t, t + 1, J, J + 1))) return st;
      } else if ((st = block(t, t + 1, 0, nj))) {
        return st;
      }
    }
    if (t < panels) {
      const int j0 = cb[t], cols = (t + 1 < panels ? cb[t + 1] : pb.Np) - j0;
      VCPCU_CUDA_TRY(cudaStreamWaitEvent(s, evB[t], 0));
      if ((st = oz_prepare_right_crt(pb, dB, k > 0 ? k : 1, ws, s, j0, cols,
                                     (size_t)pb.Np * pb.Kp)))
        return st;
      const int ni = t + 1 < row_panels ? t + 1 : row_panels;
      if (last_is_b && t == panels - 1) {
        for (int I = 0; I < ni; ++I)
          if ((st = block(I, I + 1, t, t + 1))) return st;
      } else if ((st = block(0, ni, t, t + 1))) {
        return st;
      }
    }
  }
  oz_profile_add_flops(flops);
  if ((st = pipe_event(g, c0, s)) || (st = pipe_event(g, c1, s))) return st;
  oz_merge_status(ws.flag, s);
  // A non-finite entry seen late leaves earlier blocks finite; the whole
  // result is NaN then, as in the one-shot product.
  int hflag[2] = {0, 0};
  VCPCU_CUDA_TRY(cudaMemcpyAsync(hflag, ws.flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(down));
  if ((hflag[0] != 0 || hflag[1] != 0) && panels * row_panels > 1) {
    oz_fill_nan<<<152 * 8, 256, 0, s>>>(nc, dC);
    VCPCU_LAUNCH_CHECK("oz_fill_nan");
    VCPCU_CUDA_TRY(cudaMemcpyAsync(C, dC, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
    VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return VCPCU_OK;
}

int ozaki_igemm(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                double* C, long ldc, int form, int slices, cudaStream_t s, int point_mask) {
  const int nslices = slices > 0 ? slices : 8;
  const int sr = 2;
  if (k > (1 << 20)) {
    set_error("igemm (Ozaki form): inner dimension %d above the supported 2^20", k);
    return VCPCU_ERR_UNSUPPORTED;
  }
  OzPlan plan;
  oz_make_plan(m, n, k, nslices, sr, &plan, form == VCPCU_FORM_OZAKI_SLICES ? 0 : 1);
  plan.point_mask = point_mask & 3;
  Scratch buf;
  int st = buf.alloc(oz_workspace_bytes(plan.pb), s);
  if (st) return st;
  OzWorkspace ws;
  oz_carve_workspace(plan.pb, buf.ptr, &ws);
  if ((st = oz_run_product(plan, ws, A, lda, B, ldb, C, ldc, s))) return st;
  oz_profile_add_flops(2LL * m * n * (long long)(k > 0 ? k : 0) *
                       ((plan.pb.crt ? plan.pb.L : plan.mid.npairs) +
                        (long long)(!(point_mask & 2) + !(point_mask & 1)) * plan.rad.npairs));
  oz_status_merge<<<1, 1, 0, s>>>(ws.flag);
  VCPCU_LAUNCH_CHECK("oz_status_merge");
  return VCPCU_OK;
}

}  // namespace vcpcu
