// ozaki_group.cu -- grouped CRT-form interval products (the tensor-core path
// of a batch of uneven products, vcpcu_igemm_batched_dev / the batch
// graphs).
//
// The problems of a batch are bucketed by their padded inner dimension Kp,
// modulus count L and operand width w (one CRT plan per bucket), and each
// bucket is cut into chunks of about 0.4 ms of estimated work, so that a
// problem's latency -- the length of its chunk -- stays short.  A chunk runs
// in a fixed number of launches whatever its size: row maxima, exponents,
// left and right splits, the two radius slice GEMMs, the residue slice GEMM,
// the reassembly and the status merge -- each a grouped twin of the
// single-product kernel that finds its problem through a prefix array of
// blocks or work items, or one load from an item -> problem table (the slice
// GEMM's work items are the (problem, group, tile) triples of the chunk).
// The results are bit for bit those of one vcpcu_igemm_dev call per problem:
// the same plan (w, L, moduli, digit pairs, folds) and the same arithmetic
// per entry.  Chunks run one after another on the stream and share one
// workspace (the largest chunk's); their tables (problem descriptors,
// prefix arrays) are built on the host and uploaded once by oz_group_plan.
#include "common.cuh"
#include "ozaki.cuh"
#include "ozaki_common.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

namespace vcpcu {

namespace {

size_t al256g(size_t x) { return (x + 255) & ~(size_t)255; }

struct BucketHost {
  OzGBucket dev;  // table pointers set at plan time, workspace pointers at record time
  OzPlan shape;   // radius pair list, Lmax-modulus pair list, fold count
  OzRadConst rc;
  int nblk_rowmax = 0, nblk_split = 0, nitem_rad = 0, nitem_crt = 0, nblk_asm = 0;
  int wmax = 0;  // largest operand width w of the bucket's problems
  // workspace layout (byte offsets; the first zero_bytes are cleared per run)
  size_t offRowmax = 0, offAsum = 0, offFlag = 0, zero_bytes = 0;
  size_t offE3 = 0, offF2 = 0, offBeta = 0, offA = 0, offB = 0, offRes = 0, offP = 0;
  size_t offMidB = 0, offRadB = 0, offBsum = 0, offMidA = 0, offRadA = 0;
  size_t ws_bytes = 0;
};

}  // namespace

struct OzGroupPlan {
  std::vector<BucketHost> buckets;
  void* tables = nullptr;
  void* ws = nullptr;
  size_t ws_bytes = 0;  // one workspace (the largest chunk's); nws of them at ws
  int nws = 1;
  int persistent = 0;
};

namespace {
// Work of one bucket (chunk) of the batch, estimated device time in ns.
constexpr double OZ_GROUP_CHUNK_NS = 400000.0;

// Estimated device time of one problem of a bucket (ns), from the rates the
// grouped kernels reach on GB300: about 9 ns per k-block (64) of one work
// item of the slice GEMM (L residue GEMMs and 2 x 3 radius digit pairs per
// tile), 25 ps per
// padded operand entry of the preparation, 27 ps per output entry of the
// reassembly.  Used only to cut buckets into chunks of similar length.
double group_cost_ns(const BatchProblemView& q, const OzPlan& pl) {
  const double tiles = (double)(pl.pb.Mp / OZ_BM) * (pl.pb.Np / OZ_BN);
  return 9.0 * (pl.pb.L + 2 * pl.rad.npairs) * tiles * (pl.pb.Kp / OZ_BK) +
         0.025 * ((double)pl.pb.Mp + pl.pb.Np) * pl.pb.Kp + 0.027 * (double)q.m * q.n;
}
}  // namespace

int oz_group_plan(int count, const BatchProblemView* problems, const char* select, int slices,
                  int persistent, cudaStream_t s, OzGroupPlan** out) {
  *out = nullptr;
  const int nslices = slices > 0 ? slices : 8;
  // bucket the selected problems by (Kp, L, w, radius pairs): the problems
  // of a bucket share one CRT plan (moduli, basis, digit pairs, folds)
  std::map<std::tuple<int, int, int, int>, std::vector<int>> byKey;
  std::vector<OzPlan> plans(count);
  for (int i = 0; i < count; ++i) {
    const BatchProblemView& q = problems[i];
    if ((select && !select[i]) || q.m <= 0 || q.n <= 0 || q.k <= 0) continue;
    oz_make_plan(q.m, q.n, q.k, nslices, 2, &plans[i], 1);
    byKey[std::make_tuple(plans[i].pb.Kp, plans[i].pb.L, plans[i].pb.w, plans[i].rad.npairs)]
        .push_back(i);
  }
  // A bucket runs its kernels one after another, so a problem's latency is
  // its bucket's length: each is cut into chunks of about OZ_GROUP_CHUNK_NS
  // of estimated work (every chunk is a bucket of its own; the kernels of a
  // chunk still fill the GPU).
  std::vector<std::vector<int>> chunks;
  for (auto& kv : byKey) {
    const std::vector<int>& ids = kv.second;
    double total = 0.0;
    for (int id : ids) total += group_cost_ns(problems[id], plans[id]);
    const int nch = std::max(1, (int)std::ceil(total / OZ_GROUP_CHUNK_NS));
    const double target = total / nch;
    std::vector<int> cur;
    double acc = 0.0;
    for (int id : ids) {
      const double c = group_cost_ns(problems[id], plans[id]);
      if (!cur.empty() && acc + 0.5 * c > target) {
        chunks.push_back(std::move(cur));
        cur.clear();
        acc = 0.0;
      }
      cur.push_back(id);
      acc += c;
    }
    if (!cur.empty()) chunks.push_back(std::move(cur));
  }
  OzGroupPlan* g = new OzGroupPlan();
  g->persistent = persistent;
  std::vector<uint8_t> host;  // all tables, each part 256-byte aligned
  auto reserve = [&](size_t bytes) {
    const size_t off = al256g(host.size());
    host.resize(off + bytes);
    return off;
  };
  struct Offs { size_t probs, brow, bspl, irad, icrt, basm, cols, prad, pcrt, pasm; };
  std::vector<Offs> toff;
  for (const std::vector<int>& ids : chunks) {
    const int n = (int)ids.size();
    BucketHost b;
    memset(&b.dev, 0, sizeof(b.dev));
    const OzPlan& p0 = plans[ids[0]];
    const int Kp = p0.pb.Kp;
    b.shape = p0;
    b.dev.nprob = n;
    b.dev.Kp = Kp;
    int Lmax = 0;
    long long Mtot = 0, Ntot = 0;
    for (int id : ids) {
      Lmax = std::max(Lmax, plans[id].pb.L);
      Mtot += plans[id].pb.Mp;
      Ntot += plans[id].pb.Np;
    }
    // every modulus a group of its own, Lmax of them (a problem uses its first L)
    OzPairList& crt = b.shape.crt;
    memset(&crt, 0, sizeof(crt));
    for (int l = 0; l < Lmax; ++l) {
      crt.pa[l] = crt.pb[l] = (int8_t)l;
      crt.gstart[l] = (int16_t)l;
      crt.gt[l] = (int8_t)l;
    }
    crt.gstart[Lmax] = (int16_t)Lmax;
    crt.npairs = crt.ngroups = Lmax;
    b.shape.point_mask = 0;
    b.rc = oz_rad_const(b.shape);
    b.dev.Lmax = Lmax;
    Offs o;
    o.probs = reserve(sizeof(OzGProb) * n);
    o.brow = reserve(sizeof(int) * (n + 1));
    o.bspl = reserve(sizeof(int) * (n + 1));
    o.irad = reserve(sizeof(int) * (n + 1));
    o.icrt = reserve(sizeof(int) * (n + 1));
    o.basm = reserve(sizeof(int) * (n + 1));
    o.cols = reserve(sizeof(int) * (size_t)Ntot);
    long long brow = 0, bspl = 0, irad = 0, icrt = 0, basm = 0, res = 0, P = 0;
    int rowoff = 0, coloff = 0;
    for (int t = 0; t < n; ++t) {
      const int id = ids[t];
      const BatchProblemView& q = problems[id];
      const OzPlan& pl = plans[id];
      OzGProb gp;
      memset(&gp, 0, sizeof(gp));
      gp.m = q.m;
      gp.n = q.n;
      gp.k = q.k;
      gp.A = q.A;
      gp.lda = q.lda;
      gp.B = q.B;
      gp.ldb = q.ldb;
      gp.C = q.C;
      gp.ldc = q.ldc;
      gp.Mp = pl.pb.Mp;
      gp.Np = pl.pb.Np;
      gp.L = pl.pb.L;
      gp.w = pl.pb.w;
      b.wmax = std::max(b.wmax, gp.w);
      gp.rowoff = rowoff;
      gp.coloff = coloff;
      gp.tiles_m = pl.pb.Mp / OZ_BM;
      gp.tiles_n = pl.pb.Np / OZ_BN;
      gp.res_off = res;
      gp.P_off = P;
      gp.orig = id;
      for (int l = 0; l < 16; ++l)
        for (int c = 0; c < 4; ++c) gp.Q[l][c] = l < pl.pb.L ? pl.Q[l][c] : 0u;
      for (int c = 0; c < 4; ++c) gp.Mlimb[c] = pl.Mlimb[c];
      const double Md = (double)pl.Mlimb[3] * 0x1p96 + (double)pl.Mlimb[2] * 0x1p64 +
                        (double)pl.Mlimb[1] * 0x1p32 + (double)pl.Mlimb[0];
      gp.invMf = (float)(0x1p64 / Md);
      memcpy(host.data() + o.probs + sizeof(OzGProb) * t, &gp, sizeof(gp));
      int* v;
      v = (int*)(host.data() + o.brow); v[t] = (int)brow;
      v = (int*)(host.data() + o.bspl); v[t] = (int)bspl;
      v = (int*)(host.data() + o.irad); v[t] = (int)irad;
      v = (int*)(host.data() + o.icrt); v[t] = (int)icrt;
      v = (int*)(host.data() + o.basm); v[t] = (int)basm;
      int* cols = (int*)(host.data() + o.cols);
      for (int j = 0; j < gp.Np; ++j) cols[coloff + j] = t;
      const long long tiles = (long long)gp.tiles_m * gp.tiles_n;
      brow += (long long)((q.m + 31) / 32) * ((q.k + 255) / 256);
      bspl += (long long)(Kp / 64) * (gp.Mp / 32);
      irad += b.shape.rad.ngroups * tiles;
      icrt += gp.L * tiles;
      basm += (((long long)(q.m + 3) / 4) * ((q.n + 7) / 8) + 255) / 256;
      res += (long long)gp.L * gp.Np * gp.Mp;
      P += 2LL * b.shape.rad_slots * gp.Np * gp.Mp;
      rowoff += gp.Mp;
      coloff += gp.Np;
    }
    if (std::max({brow, bspl, irad, icrt, basm}) >= INT_MAX || Mtot >= INT_MAX ||
        Ntot >= INT_MAX) {
      delete g;
      set_error("igemm_batched: the tensor-core batch is too large for one group");
      return VCPCU_ERR_INVALID_ARG;
    }
    int* v;
    v = (int*)(host.data() + o.brow); v[n] = (int)brow;
    v = (int*)(host.data() + o.bspl); v[n] = (int)bspl;
    v = (int*)(host.data() + o.irad); v[n] = (int)irad;
    v = (int*)(host.data() + o.icrt); v[n] = (int)icrt;
    v = (int*)(host.data() + o.basm); v[n] = (int)basm;
    b.nblk_rowmax = (int)brow;
    b.nblk_split = (int)bspl;
    b.nitem_rad = (int)irad;
    b.nitem_crt = (int)icrt;
    // item -> problem maps of the two kinds of slice GEMM launches (one load
    // per work item instead of a binary search over the prefixes above)
    o.prad = reserve(sizeof(int) * (size_t)(irad > 0 ? irad : 1));
    o.pcrt = reserve(sizeof(int) * (size_t)(icrt > 0 ? icrt : 1));
    o.pasm = reserve(sizeof(int) * (size_t)(basm > 0 ? basm : 1));
    {
      const int* pr = (const int*)(host.data() + o.irad);
      const int* pc = (const int*)(host.data() + o.icrt);
      const int* pa = (const int*)(host.data() + o.basm);
      int* mr = (int*)(host.data() + o.prad);
      int* mc = (int*)(host.data() + o.pcrt);
      int* ma = (int*)(host.data() + o.pasm);
      for (int t = 0; t < n; ++t) {
        for (int it = pr[t]; it < pr[t + 1]; ++it) mr[it] = t;
        for (int it = pc[t]; it < pc[t + 1]; ++it) mc[it] = t;
        for (int it = pa[t]; it < pa[t + 1]; ++it) ma[it] = t;
      }
    }
    b.nblk_asm = (int)basm;
    b.dev.Mtot = (int)Mtot;
    b.dev.Ntot = (int)Ntot;
    // workspace layout
    size_t w = 0;
    auto take = [&](size_t bytes) {
      const size_t off = w;
      w = al256g(w + bytes);
      return off;
    };
    b.offRowmax = take(sizeof(unsigned long long) * 3 * Mtot);
    b.offAsum = take(sizeof(unsigned long long) * 4 * Mtot);
    b.offFlag = take(sizeof(int) * 4 * (size_t)n);
    b.zero_bytes = w;
    b.offE3 = take(sizeof(int) * 3 * Mtot);
    b.offF2 = take(sizeof(int) * 2 * Ntot);
    b.offBeta = take(sizeof(double) * Ntot);
    b.offMidB = take(sizeof(double) * (size_t)Ntot * Kp);
    b.offRadB = take(sizeof(double) * (size_t)Ntot * Kp);
    b.offBsum = take(sizeof(unsigned long long) * 4 * Ntot);
    b.offMidA = take(sizeof(double) * (size_t)Mtot * Kp);
    b.offRadA = take(sizeof(double) * (size_t)Mtot * Kp);
    b.offA = take(sizeof(uint16_t) * (size_t)(Lmax + 4) * Mtot * Kp);
    b.offB = take(sizeof(uint16_t) * (size_t)(Lmax + 4) * Ntot * Kp);
    b.offRes = take((size_t)res);
    b.offP = take(sizeof(int32_t) * (size_t)P);
    b.ws_bytes = w;
    g->ws_bytes = std::max(g->ws_bytes, w);
    g->buckets.push_back(b);
    toff.push_back(o);
  }
  if (g->buckets.empty()) {
    *out = g;
    return VCPCU_OK;
  }
  // device memory: the tables and one workspace per stream (chunks
  // alternate between two streams when there are several)
  g->nws = g->buckets.size() > 1 ? 2 : 1;
  cudaError_t e;
  if (persistent) {
    e = cudaMalloc(&g->tables, host.size());
    if (e == cudaSuccess) e = cudaMalloc(&g->ws, g->ws_bytes * g->nws);
  } else {
    e = cudaMallocAsync(&g->tables, host.size(), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&g->ws, g->ws_bytes * g->nws, s);
  }
  if (e != cudaSuccess) {
    oz_group_free(g, s);
    return cuda_fail(e, "igemm_batched: tensor-core workspace");
  }
  e = cudaMemcpyAsync(g->tables, host.data(), host.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // `host` is freed on return
  if (e != cudaSuccess) {
    oz_group_free(g, s);
    return cuda_fail(e, "igemm_batched: upload of the group tables");
  }
  uint8_t* tb = (uint8_t*)g->tables;
  for (size_t i = 0; i < g->buckets.size(); ++i) {
    OzGBucket& d = g->buckets[i].dev;
    const Offs& o = toff[i];
    d.probs = (const OzGProb*)(tb + o.probs);
    d.blk_rowmax = (const int*)(tb + o.brow);
    d.blk_split = (const int*)(tb + o.bspl);
    d.item_rad = (const int*)(tb + o.irad);
    d.item_crt = (const int*)(tb + o.icrt);
    d.prob_rad = (const int*)(tb + o.prad);
    d.prob_crt = (const int*)(tb + o.pcrt);
    d.blk_asm = (const int*)(tb + o.basm);
    d.prob_asm = (const int*)(tb + o.pasm);
    d.col_prob = (const int*)(tb + o.cols);
  }
  *out = g;
  return VCPCU_OK;
}

namespace {
// The launches of one chunk on stream s over workspace ws.
int record_chunk(const BucketHost& b, uint8_t* ws, unsigned long long* t_first,
                 unsigned long long* t_last, cudaStream_t s) {
  OzGBucket d = b.dev;
  d.rowmax = (unsigned long long*)(ws + b.offRowmax);
  d.asum = (unsigned long long*)(ws + b.offAsum);
  d.flag = (int*)(ws + b.offFlag);
  d.E3 = (int*)(ws + b.offE3);
  d.F2 = (int*)(ws + b.offF2);
  d.beta = (double*)(ws + b.offBeta);
  d.midB = (double*)(ws + b.offMidB);
  d.radB = (double*)(ws + b.offRadB);
  d.bsum = (unsigned long long*)(ws + b.offBsum);
  d.midA = (double*)(ws + b.offMidA);
  d.radA = (double*)(ws + b.offRadA);
  d.planesA = (uint16_t*)(ws + b.offA);
  d.planesB = (uint16_t*)(ws + b.offB);
  d.res = ws + b.offRes;
  d.P = (int32_t*)(ws + b.offP);
  d.t_first = t_first;
  d.t_last = t_last;
  // (the caller resets every problem's stamps once per batch)
  VCPCU_CUDA_TRY(cudaMemsetAsync(ws, 0, b.zero_bytes, s));
  int st;
  {
    PhaseTimer t(0, s);
    if ((st = oz_gprep(d, b.nblk_rowmax, b.nblk_split, b.wmax, s))) return st;
  }
  {
    PhaseTimer t(1, s);
    if ((st = oz_grun_gemm(d, b.shape, OZ_RAD_SET, b.nitem_rad, s))) return st;
  }
  {
    PhaseTimer t(2, s);
    if ((st = oz_grun_gemm(d, b.shape, OZ_RAD_ADD, b.nitem_rad, s))) return st;
  }
  {
    PhaseTimer t(3, s);
    if ((st = oz_grun_gemm(d, b.shape, OZ_CRT, b.nitem_crt, s))) return st;
  }
  {
    PhaseTimer t(4, s);  // the reassembly also merges the chunk's status words
    if ((st = oz_gassemble(d, b.shape, b.rc, b.nblk_asm, s))) return st;
  }
  return VCPCU_OK;
}
}  // namespace

// Chunks alternate between s and a second stream forked from it, each with
// its own workspace: the launches of one chunk fill the drain tails of the
// other (a chunk's kernels run one after another and each ends in a partial
// wave).  The second stream rejoins s at the end, also after an error (a
// stream capture must end joined).
int oz_group_record(OzGroupPlan* g, unsigned long long* t_first, unsigned long long* t_last,
                    cudaStream_t s) {
  uint8_t* ws = (uint8_t*)g->ws;
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  const bool two = g->nws == 2;
  if (two) {
    cudaError_t e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(fork_ev, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side, fork_ev, 0);
    if (e != cudaSuccess) {
      if (join_ev) cudaEventDestroy(join_ev);
      if (fork_ev) cudaEventDestroy(fork_ev);
      if (side) cudaStreamDestroy(side);
      return cuda_fail(e, "igemm_batched: second stream of the tensor-core chunks");
    }
  }
  int st = VCPCU_OK;
  for (size_t i = 0; i < g->buckets.size() && !st; ++i) {
    const bool odd = two && (i & 1);
    st = record_chunk(g->buckets[i], ws + (odd ? g->ws_bytes : 0), t_first, t_last,
                      odd ? side : s);
  }
  if (two) {
    cudaEventRecord(join_ev, side);
    cudaStreamWaitEvent(s, join_ev, 0);
    cudaEventDestroy(join_ev);
    cudaEventDestroy(fork_ev);
    cudaStreamDestroy(side);
  }
  return st;
}

void oz_group_free(OzGroupPlan* g, cudaStream_t s) {
  if (!g) return;
  if (g->persistent) {
    if (g->tables) cudaFree(g->tables);
    if (g->ws) cudaFree(g->ws);
  } else {
    if (g->tables) cudaFreeAsync(g->tables, s);
    if (g->ws) cudaFreeAsync(g->ws, s);
  }
  delete g;
}

}  // namespace vcpcu
