// batch.cu -- thousands of independent interval GEMMs of uneven shapes.
//
// The calls that Newton / verification steps and Legendre_Bases_Generator
// emit are many small products of different shapes.  One persistent grouped
// kernel runs them all: each CTA takes 64 x 64 output tiles from a global
// work counter (atomicAdd; no CTA ever waits on another), finds the tile's
// problem by binary search over the tiles' prefix sums, and computes it with
// the plain-form chains of pidblas::mulmm (vcp/pidblas.hpp:239-294), midrad
// fused into the tile loads (the interval operands are read directly, no
// prep pass).  Every tile records the device clock when it starts and ends;
// per problem the first start and last end give its latency.
//
// The tensor-core (Ozaki) form runs the problems one after another on the
// stream; vcpcu_batch_graph_* capture either form into a CUDA graph so a
// batch is replayed with one launch.
#include "common.cuh"
#include "ozaki.cuh"
#include "plain_gemm.cuh"
#include "variants.cuh"

#include <algorithm>
#include <vector>

namespace vcpcu {

struct BatchProblem {  // layout mirrored by vcpcu_problem in include/vcpcuda.h
  int m, n, k;
  int lda, ldb, ldc;
  const double* A;
  const double* B;
  double* C;
};

namespace {

constexpr int BM = 64, BN = 64, BKI = 8, NT = 256;

__device__ __forceinline__ void midrad_b(double lo, double up, double& m, double& r) {
  double s = __dadd_rn(lo, up);
  if (isfinite(s))
    m = __dmul_rn(s, 0.5);
  else
    m = __dadd_rn(__dmul_rn(lo, 0.5), __dmul_rn(up, 0.5));
  r = fmax(__dsub_ru(m, lo), __dsub_ru(up, m));
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__global__ void __launch_bounds__(NT)
batched_interval_kernel(int count, const BatchProblem* __restrict__ probs,
                        const int* __restrict__ tile_start, int total_tiles,
                        int* __restrict__ counter, unsigned long long* __restrict__ t_first,
                        unsigned long long* __restrict__ t_last) {
  __shared__ double Am[BKI][BM], Ap[BKI][BM], Ar[BKI][BM];
  __shared__ double Bm[BKI][BN], Br[BKI][BN];
  __shared__ int s_tile;
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int a_i = tid % BM, a_k = tid / BM;
  const int b_k = tid % BKI, b_j = tid / BKI;
  constexpr int QA = BKI / (NT / BM), QB = BN / (NT / BKI);
  for (;;) {
    if (tid == 0) s_tile = atomicAdd(counter, 1);
    __syncthreads();
    const int tile = s_tile;
    __syncthreads();
    if (tile >= total_tiles) break;
    // problem of this tile: last p with tile_start[p] <= tile
    int lo_p = 0, hi_p = count - 1;
    while (lo_p < hi_p) {
      const int mid = (lo_p + hi_p + 1) >> 1;
      if (tile_start[mid] <= tile)
        lo_p = mid;
      else
        hi_p = mid - 1;
    }
    const BatchProblem P = probs[lo_p];
    const int local = tile - tile_start[lo_p];
    const int tm_count = (P.m + BM - 1) / BM;
    const int row0 = (local % tm_count) * BM, col0 = (local / tm_count) * BN;
    unsigned long long t0 = 0;
    if (tid == 0) t0 = gtimer();

    double lo[4][4], up[4][4], t1[4][4], t2[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) lo[i][j] = up[i][j] = t1[i][j] = t2[i][j] = 0.0;
    for (int k0 = 0; k0 < P.k; k0 += BKI) {
#pragma unroll
      for (int q = 0; q < QA; ++q) {
        const int gi = row0 + a_i, gk = k0 + a_k + (NT / BM) * q;
        double m = 0.0, r = 0.0, p = 0.0;
        if (gi < P.m && gk < P.k) {
          const double* e = P.A + 2 * (gi + (long)gk * P.lda);
          midrad_b(e[0], e[1], m, r);
          p = __dadd_ru(fabs(m), r);
        }
        Am[a_k + (NT / BM) * q][a_i] = m;
        Ap[a_k + (NT / BM) * q][a_i] = p;
        Ar[a_k + (NT / BM) * q][a_i] = r;
      }
#pragma unroll
      for (int q = 0; q < QB; ++q) {
        const int hk = k0 + b_k, hj = col0 + b_j + (NT / BKI) * q;
        double m = 0.0, r = 0.0;
        if (hk < P.k && hj < P.n) {
          const double* e = P.B + 2 * (hk + (long)hj * P.ldb);
          midrad_b(e[0], e[1], m, r);
        }
        Bm[b_k][b_j + (NT / BKI) * q] = m;
        Br[b_k][b_j + (NT / BKI) * q] = r;
      }
      __syncthreads();
#pragma unroll 2
      for (int kk = 0; kk < BKI; ++kk) {
        double am[4], ap[4], ar[4], bm[4], br[4], bma[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          am[i] = Am[kk][tr + 16 * i];
          ap[i] = Ap[kk][tr + 16 * i];
          ar[i] = Ar[kk][tr + 16 * i];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          bm[j] = Bm[kk][tc + 16 * j];
          br[j] = Br[kk][tc + 16 * j];
          bma[j] = fabs(bm[j]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            lo[i][j] = __fma_rd(am[i], bm[j], lo[i][j]);
            up[i][j] = __fma_ru(am[i], bm[j], up[i][j]);
            t1[i][j] = __fma_ru(ap[i], br[j], t1[i][j]);
            t2[i][j] = __fma_ru(ar[i], bma[j], t2[i][j]);
          }
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int gi = row0 + tr + 16 * i, gj = col0 + tc + 16 * j;
        if (gi < P.m && gj < P.n) {
          const double T = __dadd_ru(t1[i][j], t2[i][j]);
          double* e = P.C + 2 * (gi + (long)gj * P.ldc);
          e[0] = __dsub_rd(lo[i][j], T);
          e[1] = __dadd_ru(up[i][j], T);
        }
      }
    if (tid == 0 && t_first) {
      atomicMin(&t_first[lo_p], t0);
      atomicMax(&t_last[lo_p], gtimer());
    }
  }
}

__global__ void fill_u64(unsigned long long* p, int n, unsigned long long v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

}  // namespace

// Device-side batch state (problem table, tile prefix sums, counter,
// timestamps) in one stream-ordered allocation owned by the caller.
struct BatchDev {
  BatchProblem* probs;
  int* tile_start;
  int* counter;
  unsigned long long* t_first;
  unsigned long long* t_last;
  int count, total_tiles;
};

size_t batch_state_bytes(int count) {
  return round_up(sizeof(BatchProblem) * count, 256) + round_up(sizeof(int) * (count + 1), 256) +
         256 + 2 * round_up(sizeof(unsigned long long) * count, 256);
}

int batch_upload(int count, const BatchProblem* host_probs, void* mem, BatchDev* d,
                 cudaStream_t s, std::vector<int>* tiles_host) {
  uint8_t* p = (uint8_t*)mem;
  d->probs = (BatchProblem*)p;
  p += round_up(sizeof(BatchProblem) * count, 256);
  d->tile_start = (int*)p;
  p += round_up(sizeof(int) * (count + 1), 256);
  d->counter = (int*)p;
  p += 256;
  d->t_first = (unsigned long long*)p;
  p += round_up(sizeof(unsigned long long) * count, 256);
  d->t_last = (unsigned long long*)p;
  d->count = count;
  std::vector<int>& ts = *tiles_host;
  ts.assign(count + 1, 0);
  long total = 0;
  for (int i = 0; i < count; ++i) {
    ts[i] = (int)total;
    const BatchProblem& q = host_probs[i];
    if (q.m > 0 && q.n > 0) total += (long)((q.m + BM - 1) / BM) * ((q.n + BN - 1) / BN);
  }
  if (total > 0x7fffffff) {
    set_error("batched igemm: more than 2^31 tiles");
    return VCPCU_ERR_INVALID_ARG;
  }
  ts[count] = (int)total;
  d->total_tiles = (int)total;
  VCPCU_CUDA_TRY(cudaMemcpyAsync(d->probs, host_probs, sizeof(BatchProblem) * count,
                                 cudaMemcpyHostToDevice, s));
  VCPCU_CUDA_TRY(cudaMemcpyAsync(d->tile_start, ts.data(), sizeof(int) * (count + 1),
                                 cudaMemcpyHostToDevice, s));
  return VCPCU_OK;
}

// One grouped launch of the plain form (reset of the counter and the
// timestamps included), stream-ordered and capturable.
int batch_reset_stamps(const BatchDev& d, cudaStream_t s) {
  fill_u64<<<(d.count + 255) / 256, 256, 0, s>>>(d.t_first, d.count, ~0ULL);
  VCPCU_LAUNCH_CHECK("fill_u64");
  fill_u64<<<(d.count + 255) / 256, 256, 0, s>>>(d.t_last, d.count, 0ULL);
  VCPCU_LAUNCH_CHECK("fill_u64");
  return VCPCU_OK;
}

int batch_launch_plain(const BatchDev& d, cudaStream_t s, bool reset = true) {
  VCPCU_CUDA_TRY(cudaMemsetAsync(d.counter, 0, sizeof(int), s));
  if (reset) {
    int st = batch_reset_stamps(d, s);
    if (st) return st;
  }
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms;  // one resident CTA per SM (about 200 registers per thread)
  if (d.total_tiles < grid) grid = d.total_tiles > 0 ? d.total_tiles : 1;
  batched_interval_kernel<<<grid, NT, 0, s>>>(d.count, d.probs, d.tile_start, d.total_tiles,
                                              d.counter, d.t_first, d.t_last);
  VCPCU_LAUNCH_CHECK("batched_interval_kernel");
  return VCPCU_OK;
}

}  // namespace vcpcu

// ---------------------------------------------------------------- C ABI
namespace vcpcu {
namespace {

__global__ void stamp(unsigned long long* p) { *p = gtimer(); }

struct BatchGraph {
  int count = 0, form = 0, slices = 0;
  OzGroupPlan* group = nullptr;  // CRT / AUTO: the grouped tensor-core products
  std::vector<BatchProblem> probs;
  std::vector<int> tiles;
  std::vector<char> ozaki;  // AUTO: problem runs in the tensor-core form
  void* state = nullptr;  // device: BatchDev arrays
  BatchDev d{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

// Tensor-core forms: every selected problem is one product (preparation,
// slice GEMMs, reassembly) bracketed by device clock stamps (t_first /
// t_last).  The products are spread round-robin over OZ_BATCH_STREAMS
// streams forked from `s` and joined back into it, so the small products of
// a batch overlap on the GPU (inside a capture the branches become parallel
// graph branches).
constexpr int OZ_BATCH_STREAMS = 16;

// Forked branches of one batch: created by fork(), joined back into the
// parent stream by join().
struct Branches {
  cudaStream_t side[OZ_BATCH_STREAMS];
  cudaEvent_t join_ev[OZ_BATCH_STREAMS];
  int made = 0;

  int fork(cudaStream_t s, int want) {
    cudaEvent_t f;
    VCPCU_CUDA_TRY(cudaEventCreateWithFlags(&f, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(f, s);
    for (; e == cudaSuccess && made < want; ++made) {
      e = cudaStreamCreateWithFlags(&side[made], cudaStreamNonBlocking);
      if (e != cudaSuccess) break;
      e = cudaEventCreateWithFlags(&join_ev[made], cudaEventDisableTiming);
      if (e != cudaSuccess) {
        cudaStreamDestroy(side[made]);
        break;
      }
      e = cudaStreamWaitEvent(side[made], f, 0);
    }
    cudaEventDestroy(f);
    return e == cudaSuccess ? VCPCU_OK : cuda_fail(e, "batch: fork streams");
  }
  // every branch rejoins s (also after an error: a capture must end joined)
  void join(cudaStream_t s) {
    for (int b = 0; b < made; ++b) {
      cudaEventRecord(join_ev[b], side[b]);
      cudaStreamWaitEvent(s, join_ev[b], 0);
      cudaEventDestroy(join_ev[b]);
      cudaStreamDestroy(side[b]);
    }
    made = 0;
  }
};

// The selected problems round-robin over the branches, each bracketed by
// its stamps.
int batch_issue_ozaki(const BatchGraph& g, Branches& br, bool auto_only) {
  int r = 0;
  for (int i = 0; i < g.count; ++i) {
    const BatchProblem& q = g.probs[i];
    const bool run = q.m > 0 && q.n > 0 && (!auto_only || g.ozaki[i]);
    if (auto_only && !run) continue;
    cudaStream_t t = br.side[r++ % br.made];
    stamp<<<1, 1, 0, t>>>(g.d.t_first + i);
    if (run) {
      const int st = igemm_any(q.m, q.n, q.k > 0 ? q.k : 0, q.A, q.lda, q.B, q.ldb, q.C, q.ldc,
                               auto_only ? VCPCU_FORM_OZAKI : g.form, g.slices, t);
      if (st) return st;
    }
    stamp<<<1, 1, 0, t>>>(g.d.t_last + i);
  }
  VCPCU_LAUNCH_CHECK("stamp");
  return VCPCU_OK;
}

int batch_record(BatchGraph& g, cudaStream_t s) {
  if (g.form == VCPCU_FORM_PLAIN) return batch_launch_plain(g.d, s);
  if (g.form == VCPCU_FORM_OZAKI_SLICES) {  // product by product on forked streams
    Branches br;
    int st = br.fork(s, g.count < OZ_BATCH_STREAMS ? g.count : OZ_BATCH_STREAMS);
    if (!st) st = batch_issue_ozaki(g, br, false);
    br.join(s);
    return st;
  }
  // CRT form and AUTO: the tensor-core problems as grouped products on s;
  // AUTO's plain problems in the grouped plain launch on a forked branch
  const bool is_auto = g.form == VCPCU_FORM_AUTO;
  int st = batch_reset_stamps(g.d, s);
  if (st) return st;
  Branches br;
  if (is_auto) {
    if ((st = br.fork(s, 1))) {
      br.join(s);
      return st;
    }
    st = batch_launch_plain(g.d, br.side[0], false);
  }
  // tensor-core problems outside the groups (k == 0) one by one
  for (int i = 0; i < g.count && !st; ++i) {
    const BatchProblem& q = g.probs[i];
    if (q.m <= 0 || q.n <= 0 || q.k > 0 || (is_auto && !g.ozaki[i])) continue;
    stamp<<<1, 1, 0, s>>>(g.d.t_first + i);
    st = igemm_any(q.m, q.n, 0, q.A, q.lda, q.B, q.ldb, q.C, q.ldc, VCPCU_FORM_OZAKI, g.slices,
                   s);
    stamp<<<1, 1, 0, s>>>(g.d.t_last + i);
  }
  if (!st && g.group) st = oz_group_record(g.group, g.d.t_first, g.d.t_last, s);
  br.join(s);
  return st;
}

// Leading dimensions of every problem; the tensor-core forms read the
// intervals of A and B as 16-byte pairs (AUTO sends misaligned problems to
// the plain form instead).
int batch_check(const std::vector<BatchProblem>& probs, int form) {
  for (const BatchProblem& q : probs) {
    if (q.m <= 0 || q.n <= 0) continue;
    if (q.lda < q.m || q.ldc < q.m || (q.k > 0 && q.ldb < q.k) || !q.C ||
        (q.k > 0 && (!q.A || !q.B))) {
      set_error("igemm_batched: null pointer or leading dimension too small in a problem");
      return VCPCU_ERR_INVALID_ARG;
    }
    if ((form == VCPCU_FORM_OZAKI || form == VCPCU_FORM_OZAKI_SLICES) && q.k > 0 &&
        ((((uintptr_t)q.A) | ((uintptr_t)q.B)) & 15) != 0) {
      set_error("igemm_batched: the tensor-core forms need 16-byte aligned A and B");
      return VCPCU_ERR_INVALID_ARG;
    }
  }
  return VCPCU_OK;
}

// The grouped tensor-core plan of a CRT / AUTO batch (null otherwise).
int batch_group_plan(BatchGraph& g, int persistent, cudaStream_t s) {
  if (g.form != VCPCU_FORM_OZAKI && g.form != VCPCU_FORM_AUTO) return VCPCU_OK;
  std::vector<char> sel;
  if (g.form == VCPCU_FORM_AUTO) sel = g.ozaki;
  return oz_group_plan(g.count, reinterpret_cast<const BatchProblemView*>(g.probs.data()),
                       sel.empty() ? nullptr : sel.data(), g.slices, persistent, s, &g.group);
}

// AUTO: mark the problems the autotuner sends to the tensor-core form and
// hide them from the grouped plain launch (zero tiles).
void batch_split_auto(BatchGraph& g, std::vector<BatchProblem>& plain_view) {
  g.ozaki.assign(g.count, 0);
  plain_view = g.probs;
  if (g.form != VCPCU_FORM_AUTO) return;
  for (int i = 0; i < g.count; ++i) {
    const BatchProblem& q = g.probs[i];
    if (q.m > 0 && q.n > 0 && autotune_choose(q.m, q.n, q.k > 0 ? q.k : 0, true) != VCPCU_FORM_PLAIN &&
        ((((uintptr_t)q.A) | ((uintptr_t)q.B)) & 15) == 0) {
      g.ozaki[i] = 1;
      plain_view[i].m = 0;
    }
  }
}

}  // namespace
}  // namespace vcpcu

using namespace vcpcu;

extern "C" {

int vcpcu_igemm_batched_dev(int count, const vcpcu_problem* problems, int form, int slices,
                            void* stream) {
  clear_error();
  if (count <= 0) return VCPCU_OK;
  if (!problems || (form != VCPCU_FORM_PLAIN && form != VCPCU_FORM_OZAKI &&
                    form != VCPCU_FORM_OZAKI_SLICES && form != VCPCU_FORM_AUTO)) {
    set_error("igemm_batched: null problem table or unsupported form %d", form);
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  BatchGraph g;
  g.count = count;
  g.form = form;
  g.slices = slices;
  g.probs.assign((const BatchProblem*)problems, (const BatchProblem*)problems + count);
  if ((st = batch_check(g.probs, form))) return st;
  std::vector<BatchProblem> plain_view;
  batch_split_auto(g, plain_view);
  Scratch mem;
  if ((st = mem.alloc(batch_state_bytes(count), s))) return st;
  if ((st = batch_upload(count, plain_view.data(), mem.ptr, &g.d, s, &g.tiles))) return st;
  if ((st = batch_group_plan(g, 0, s))) return st;
  st = batch_record(g, s);
  oz_group_free(g.group, s);
  return st;
}

int vcpcu_batch_graph_create(int count, const vcpcu_problem* problems, int form, int slices,
                             void* stream, vcpcu_batch_graph* out) {
  clear_error();
  if (!out || count <= 0 || !problems ||
      (form != VCPCU_FORM_PLAIN && form != VCPCU_FORM_OZAKI && form != VCPCU_FORM_OZAKI_SLICES &&
       form != VCPCU_FORM_AUTO)) {
    set_error("batch_graph_create: bad arguments");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  BatchGraph* g = new BatchGraph();
  g->count = count;
  g->form = form;
  g->slices = slices;
  g->probs.assign((const BatchProblem*)problems, (const BatchProblem*)problems + count);
  if ((st = batch_check(g->probs, form))) {
    delete g;
    return st;
  }
  std::vector<BatchProblem> plain_view;
  batch_split_auto(*g, plain_view);
  cudaError_t e = cudaMalloc(&g->state, batch_state_bytes(count));
  if (e != cudaSuccess) {
    delete g;
    return cuda_fail(e, "cudaMalloc(batch state)");
  }
  if ((st = batch_upload(count, plain_view.data(), g->state, &g->d, s, &g->tiles)) ||
      (st = batch_group_plan(*g, 1, s))) {
    oz_group_free(g->group, s);
    cudaFree(g->state);
    delete g;
    return st;
  }
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaFree(g->state);
    delete g;
    return cuda_fail(e, "cudaStreamSynchronize");
  }
  // capture one batch on a private stream
  cudaStream_t cs;
  cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    st = batch_record(*g, cs);
    cudaError_t e2 = cudaStreamEndCapture(cs, &g->graph);
    if (!st && e2 != cudaSuccess) st = cuda_fail(e2, "cudaStreamEndCapture");
    if (!st) {
      e2 = cudaGraphInstantiate(&g->exec, g->graph, 0);
      if (e2 != cudaSuccess) st = cuda_fail(e2, "cudaGraphInstantiate");
    }
  } else {
    st = cuda_fail(e, "cudaStreamBeginCapture");
  }
  cudaStreamDestroy(cs);
  if (st) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    oz_group_free(g->group, s);
    cudaFree(g->state);
    delete g;
    return st;
  }
  *out = (vcpcu_batch_graph)g;
  return VCPCU_OK;
}

int vcpcu_batch_graph_launch(vcpcu_batch_graph h, void* stream) {
  clear_error();
  if (!h) {
    set_error("batch_graph_launch: null handle");
    return VCPCU_ERR_INVALID_ARG;
  }
  BatchGraph* g = (BatchGraph*)h;
  VCPCU_CUDA_TRY(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  count_launch();
  return VCPCU_OK;
}

int vcpcu_batch_graph_latencies(vcpcu_batch_graph h, void* stream, double* start_us,
                                double* latency_us) {
  clear_error();
  if (!h) {
    set_error("batch_graph_latencies: null handle");
    return VCPCU_ERR_INVALID_ARG;
  }
  BatchGraph* g = (BatchGraph*)h;
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<unsigned long long> f(g->count), l(g->count);
  VCPCU_CUDA_TRY(cudaMemcpyAsync(f.data(), g->d.t_first, sizeof(unsigned long long) * g->count,
                                 cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaMemcpyAsync(l.data(), g->d.t_last, sizeof(unsigned long long) * g->count,
                                 cudaMemcpyDeviceToHost, s));
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  unsigned long long t0 = ~0ULL;
  for (int i = 0; i < g->count; ++i)
    if (f[i] != ~0ULL && f[i] < t0) t0 = f[i];
  for (int i = 0; i < g->count; ++i) {
    const bool empty = f[i] == ~0ULL || l[i] < f[i];
    if (start_us) start_us[i] = empty ? 0.0 : (double)(f[i] - t0) * 1e-3;
    if (latency_us) latency_us[i] = empty ? 0.0 : (double)(l[i] - f[i]) * 1e-3;
  }
  return VCPCU_OK;
}

int vcpcu_batch_graph_destroy(vcpcu_batch_graph h) {
  clear_error();
  if (!h) return VCPCU_OK;
  BatchGraph* g = (BatchGraph*)h;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->state) cudaFree(g->state);
  oz_group_free(g->group, nullptr);
  delete g;
  return VCPCU_OK;
}

}  // extern "C"
