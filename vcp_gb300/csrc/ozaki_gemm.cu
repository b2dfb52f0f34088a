// ozaki_gemm.cu -- the slice GEMM of the Ozaki form on tcgen05 tensor cores.
//
// A work item is one output tile (128 x 256) and one group of digit / residue
// plane pairs (A_p, B_q).  Each pair is a bf16 GEMM over the whole (padded)
// inner dimension, split into chunks of 1024: every chunk accumulates in fp32
// in tensor memory, where it is an exact integer (|digit products| <= 2^14,
// 1024 of them <= 2^24).  Epilogue warps drain each finished chunk
// (double-buffered TMEM accumulators, so draining overlaps the next chunk's
// MMAs) and, per mode:
//   OZ_CRT       group g = modulus m_g: the residue of the integer product
//                mod m_g, one byte per entry in res[g][col][row] (one chunk:
//                reduced on the FP32 pipe straight from TMEM; several: int32
//                chunk sums, reduced per fold of 64 chunks);
//   OZ_RAD_SET / OZ_RAD_ADD  all digit pairs of one radius product form one
//                group: every chunk is weighted by its pair's 2^(8 (t_ref - t))
//                and summed upward in fp32, one fold per (product, tile) into
//                P (radius factors were rounded up, so the sum bounds them);
//   OZ_MID       (slice form) folds into an int64 fixed-point value
//                W = sum_t C_t 2^(8 (t_ref - t)) in global memory; the last
//                fold is merged into the final epilogue
//                [lo, up] = [RD(W unit) - e, RU((W + R) unit) + e].
//
// Grouped products (a batch bucket) load B in 64-row boxes and multiply only
// the 64-column blocks of a tile that hold columns of its problem (MMA N =
// 64 .. 256): a narrow problem moves and multiplies a quarter to three
// quarters of a full tile; the epilogue skips the blocks that were not
// multiplied (their columns are past N and never stored for reassembly).
//
// Warp roles (320 threads, one CTA per SM, persistent over tiles):
//   warp 0      TMA producer (4-stage ring of 48 KB A+B k-blocks)
//   warp 1      TMEM owner + MMA issuer (one thread)
//   warps 2..9  epilogue: warp w reads TMEM lanes 32*(w%4).. and columns
//               128*((w-2)/4).. of each accumulator.
// Every mbarrier wait is bounded; a timeout sets flag[1] and the CTA winds
// down (waits for its copies and MMAs, frees TMEM, returns).
#include "common.cuh"
#include "ozaki.cuh"
#include "ozaki_common.cuh"
#include "swfp.cuh"
#include "tc_ptx.cuh"

#include <mutex>

namespace vcpcu {

namespace {

constexpr int NTHREADS = 320;
constexpr int A_STAGE = OZ_BM * OZ_BK * 2;  // 16 KB
constexpr int B_STAGE = OZ_BN * OZ_BK * 2;  // 32 KB
constexpr int B_SUB = 64 * OZ_BK * 2;       // 8 KB: one 64-column block of B
constexpr int STAGE_BYTES = A_STAGE + B_STAGE;
constexpr int TMEM_COLS = 512;  // two 128 x 256 fp32 accumulators

struct Smem {
  uint64_t full[OZ_STAGES], empty[OZ_STAGES];
  uint64_t tfull[2], tempty[2];
  uint64_t mma_done;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ void raise_timeout(Smem* sm, int* flag, int where) {
  atomicOr(&flag[1], 1 << where);
  *(volatile int*)&sm->abort = 1;
}

__device__ __forceinline__ double scale_dir(double x, int e, bool up) {
  while (e > 1023) {
    x = up ? __dmul_ru(x, 0x1p1023) : __dmul_rd(x, 0x1p1023);
    e -= 1023;
  }
  while (e < -1022) {
    x = up ? __dmul_ru(x, 0x1p-1022) : __dmul_rd(x, 0x1p-1022);
    e += 1022;
  }
  const double p = __longlong_as_double((long long)(e + 1023) << 52);
  return up ? __dmul_ru(x, p) : __dmul_rd(x, p);
}

// Smallest double >= 2^e (e may be below the subnormal range).
__device__ __forceinline__ double pow2_ru(int e) {
  if (e >= -1022) return scale_dir(1.0, e, true);
  if (e >= -1074) return __longlong_as_double(1LL << (e + 1074));
  return __longlong_as_double(1LL);
}

// Tile order: groups of OZ_RASTER row blocks, column blocks outer inside a
// group, so the CTAs resident at one time share a few A row panels and
// B column panels (both stay in L2 across the CTAs of one group).
constexpr int OZ_RASTER = 16;
__device__ __forceinline__ void tile_coords(int tile, int tiles_m, int tiles_n, int& tm, int& tn) {
  const int per_group = OZ_RASTER * tiles_n;
  const int g = tile / per_group;
  const int rows = min(OZ_RASTER, tiles_m - g * OZ_RASTER);
  const int idx = tile - g * per_group;
  tn = idx / rows;
  tm = g * OZ_RASTER + idx % rows;
}

// Work items.  MID (slice form): one item per tile, all groups (the groups
// accumulate into one W).  CRT and radius modes: one item per (group, tile),
// group-major -- every group writes its own residue plane or fold slots, so
// items are independent, and the CTAs in flight share one group's planes
// (compact L2 working set; the tail is one group of one tile).  Grouped
// products: the items of problem p follow one another, group-major within p.
struct ItemInfo {
  int arow, bcol;   // TMA row of the A tile / of the B tile in the planes
  int tm, tn, g0, g1;
  int nb;           // 64-column blocks of B the tile multiplies (1..4)
  int Mp, Np;       // output layout of this item's problem
  int M, N;         // its valid rows / columns
  uint8_t* res;
  int32_t* P;
};

__device__ __forceinline__ int gfind_item(const int* __restrict__ prefix, int nprob, int x) {
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ ItemInfo item_info(const OzGemmArgs& a, int item, int ntiles) {
  ItemInfo f;
  if (a.gp) {
    const int p = a.gprob ? a.gprob[item] : gfind_item(a.gitem, a.gnprob, item);
    const OzGProb& q = a.gp[p];
    const int nt = q.tiles_m * q.tiles_n;
    const int local = item - a.gitem[p];
    f.g0 = local / nt;
    f.g1 = f.g0 + 1;
    tile_coords(local - f.g0 * nt, q.tiles_m, q.tiles_n, f.tm, f.tn);
    f.arow = q.rowoff + f.tm * OZ_BM;
    f.bcol = q.coloff + f.tn * OZ_BN;
    f.Mp = q.Mp;
    f.Np = q.Np;
    f.M = q.m;
    f.N = q.n;
    f.nb = a.bsub ? min(4, (f.N - f.tn * OZ_BN + 63) >> 6) : 4;
    f.res = a.res ? a.res + q.res_off : nullptr;
    f.P = a.P ? a.P + q.P_off : nullptr;
    return f;
  }
  int tile = item;
  if (a.mode == OZ_MID) {
    f.g0 = 0;
    f.g1 = a.pl.ngroups;
  } else {
    f.g0 = item / ntiles;
    f.g1 = f.g0 + 1;
    tile = item - f.g0 * ntiles;
  }
  tile_coords(tile, a.tiles_m, a.tiles_n, f.tm, f.tn);
  f.arow = f.tm * OZ_BM;
  f.bcol = f.tn * OZ_BN;
  f.Mp = a.Mp;
  f.Np = a.Np;
  f.M = a.M;
  f.N = a.N;
  f.nb = 4;
  f.res = a.res;
  f.P = a.P;
  return f;
}

// Residue of a one-chunk CRT group on the FP32 pipe (no float-to-int
// conversion, which GB300 issues on its narrow XU pipe, and no integer
// reduction).  The chunk value x is an exact integer with |x| <= 2^24, so
// |RN(x RN(1/m)) - x/m| <= (2^24/m) 2^-23 (1 + 2^-25) and q = rint of it
// (the add and subtract of 1.5 2^23) is within 1/2 + 2.0000002/m of x/m:
// r = RN(q (-m) + x) (one FMA, exact) is an integer with |r| <= m/2 + 2,
// and adding m to a negative r gives [0, m) (m >= 107).  The epilogue
// evaluates it for two columns per paired FP32 instruction.

__device__ __forceinline__ long long shift_t(int c, int sh) {
  const long long v = (long long)c;
  return sh >= 0 ? (v << sh) : (v >> (-sh));
}

__global__ void __launch_bounds__(NTHREADS, 1)
oz_slice_gemm_kernel(const __grid_constant__ OzGemmArgs args) {
  extern __shared__ uint8_t dsmem_raw[];
  __shared__ Smem sm;
  uint8_t* dsmem = (uint8_t*)(((uintptr_t)dsmem_raw + 1023) & ~(uintptr_t)1023);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = args.tiles_m * args.tiles_n;
  const int nitems = args.gp ? args.gnitems
                             : (args.mode == OZ_MID ? ntiles : ntiles * args.pl.ngroups);
  const int nchunks = (args.Kp + OZ_CHUNK - 1) / OZ_CHUNK;
  const int kblocks = args.Kp / OZ_BK;
  const long long lim = args.timeout_cycles;

  if (threadIdx.x == 0) {
    for (int i = 0; i < OZ_STAGES; ++i) {
      ptx::mbar_init(&sm.full[i], 1);
      ptx::mbar_init(&sm.empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      ptx::mbar_init(&sm.tfull[i], 1);
      ptx::mbar_init(&sm.tempty[i], 8);
    }
    ptx::mbar_init(&sm.mma_done, 1);
    sm.abort = 0;
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc(&sm.tmem_base, TMEM_COLS);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = sm.tmem_base;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      ptx::prefetch_tmap(&args.tmA);
      ptx::prefetch_tmap(&args.tmB);
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      uint32_t used = 0, lastpar = 0;  // per-stage bit masks
      for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
        const ItemInfo f = item_info(args, item, ntiles);
        for (int pi = args.pl.gstart[f.g0]; pi < args.pl.gstart[f.g1] && ok; ++pi) {
          const int pa = args.pl.pa[pi], pb = args.pl.pb[pi];
          for (int kb = 0; kb < kblocks; ++kb) {
            if (*(volatile int*)&sm.abort || !ptx::mbar_wait(&sm.empty[stage], phase ^ 1, lim)) {
              if (!*(volatile int*)&sm.abort) raise_timeout(&sm, args.flag, 0);
              ok = false;
              break;
            }
            uint8_t* sA = dsmem + stage * STAGE_BYTES;
            uint8_t* sB = sA + A_STAGE;
            ptx::mbar_expect_tx(&sm.full[stage], A_STAGE + f.nb * B_SUB);
            ptx::tma_load_3d(sA, &args.tmA, &sm.full[stage], kb * OZ_BK, f.arow, pa);
            if (args.bsub) {
              // 64-row boxes land back to back: the same SW128 K-major
              // layout as one box of 64 nb rows
              for (int i = 0; i < f.nb; ++i)
                ptx::tma_load_3d(sB + i * B_SUB, &args.tmB, &sm.full[stage], kb * OZ_BK,
                                 f.bcol + 64 * i, pb);
            } else {
              ptx::tma_load_3d(sB, &args.tmB, &sm.full[stage], kb * OZ_BK, f.bcol, pb);
            }
            used |= 1u << stage;
            lastpar = (lastpar & ~(1u << stage)) | (phase << stage);
            if (++stage == OZ_STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      // every issued copy has landed before the CTA may exit (immediate in
      // the normal case: the MMA thread consumed them all)
      for (int i = 0; i < OZ_STAGES; ++i)
        if (used & (1u << i)) ptx::mbar_wait(&sm.full[i], (lastpar >> i) & 1u, lim);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      uint32_t acc = 0;  // global chunk counter
      bool ok = true;
      for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
        const ItemInfo f = item_info(args, item, ntiles);
        const uint32_t idesc = ptx::idesc_bf16_f32(OZ_BM, 64 * f.nb);
        for (int pi = args.pl.gstart[f.g0]; pi < args.pl.gstart[f.g1] && ok; ++pi) {
          for (int ch = 0; ch < nchunks && ok; ++ch, ++acc) {
            const int buf = acc & 1;
            const uint32_t par = (acc >> 1) & 1;
            if (*(volatile int*)&sm.abort || !ptx::mbar_wait(&sm.tempty[buf], par ^ 1, lim)) {
              if (!*(volatile int*)&sm.abort) raise_timeout(&sm, args.flag, 1);
              ok = false;
              break;
            }
            ptx::tc_fence_after();
            const uint32_t dt = tmem + buf * OZ_BN;
            const int kb0 = ch * (OZ_CHUNK / OZ_BK);
            const int kb1 = min(kblocks, kb0 + OZ_CHUNK / OZ_BK);
            for (int kb = kb0; kb < kb1; ++kb) {
              if (*(volatile int*)&sm.abort || !ptx::mbar_wait(&sm.full[stage], phase, lim)) {
                if (!*(volatile int*)&sm.abort) raise_timeout(&sm, args.flag, 2);
                ok = false;
                break;
              }
              ptx::tc_fence_after();
              const uint32_t sA = ptx::smem_u32(dsmem + stage * STAGE_BYTES);
              const uint32_t sB = sA + A_STAGE;
#pragma unroll
              for (int kk = 0; kk < OZ_BK / 16; ++kk) {
                const uint64_t ad = ptx::sw128_kmajor_desc(sA + kk * 32);
                const uint64_t bd = ptx::sw128_kmajor_desc(sB + kk * 32);
                ptx::mma_bf16(dt, ad, bd, idesc, (kb > kb0 || kk > 0) ? 1u : 0u);
              }
              ptx::mma_commit(&sm.empty[stage]);
              if (++stage == OZ_STAGES) {
                stage = 0;
                phase ^= 1;
              }
            }
            if (!ok) break;
            ptx::mma_commit(&sm.tfull[buf]);
          }
        }
      }
      // all MMAs of this thread done before TMEM is released
      ptx::mma_commit(&sm.mma_done);
      ptx::mbar_wait(&sm.mma_done, 0, lim);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 2;
    const int quarter = warp & 3;
    const int half = ew >> 2;
    const int row_in_tile = quarter * 32 + lane;
    const uint32_t lane_addr = (uint32_t)(quarter * 32) << 16;
    uint32_t acc = 0;
    bool ok = true;
    bool nonfinite = args.flag[0] != 0;
    for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
      const ItemInfo f = item_info(args, item, ntiles);
      const int g0 = f.g0, g1 = f.g1;
      const int gi = f.tm * OZ_BM + row_in_tile;
      const int gj0 = f.tn * OZ_BN + half * 128;
      if (args.mode != OZ_MID && f.tm * OZ_BM + quarter * 32 >= f.M) {
        // this warp's 32 rows are all past M (padding of the tile): release
        // each accumulator of the item unread -- the reassembly reads no
        // padding row (midpoint folds keep every row)
        for (int g = g0; g < g1 && ok; ++g) {
          const int total = (args.gkind[g] == OZ_CRT && nchunks == 1)
                                ? 1
                                : (args.pl.gstart[g + 1] - args.pl.gstart[g]) * nchunks;
          for (int idx = 0; idx < total; ++idx, ++acc) {
            const int buf = acc & 1;
            const uint32_t par = (acc >> 1) & 1;
            if (*(volatile int*)&sm.abort || !ptx::mbar_wait(&sm.tfull[buf], par, lim)) {
              if (!*(volatile int*)&sm.abort) raise_timeout(&sm, args.flag, 3);
              ok = false;
              break;
            }
            ptx::tc_fence_after();
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&sm.tempty[buf]);
          }
        }
        continue;
      }
      bool have_w = false;
      for (int g = g0; g < g1 && ok; ++g) {
        const int kind = args.gkind[g];
        if (kind == OZ_RAD_SET || kind == OZ_RAD_ADD) {
          // radius product (its digit pairs form one group): every chunk, an
          // exact integer in fp32, is weighted by its pair's 2^(8 (t_ref - t))
          // and summed upward -- S = RU(chunk 2^sh + S), an upper bound of
          // the exact weighted integer sum -- and one fold per (product, tile)
          // goes out, never read back here
          const int ncb = (f.nb * 64 - half * 128) >> 5;  // column blocks multiplied
          float S[128];
#pragma unroll
          for (int e = 0; e < 128; ++e) S[e] = 0.0f;
          int pi = args.pl.gstart[g], pc = 0;
          const int total = (args.pl.gstart[g + 1] - pi) * nchunks;
          for (int idx = 0; idx < total; ++idx, ++acc) {
            const int buf = acc & 1;
            const uint32_t par = (acc >> 1) & 1;
            if (*(volatile int*)&sm.abort || !ptx::mbar_wait(&sm.tfull[buf], par, lim)) {
              if (!*(volatile int*)&sm.abort) raise_timeout(&sm, args.flag, 3);
              ok = false;
              break;
            }
            ptx::tc_fence_after();
            const float sc = __int_as_float((127 + 8 * (args.t_ref - args.pl.pt[pi])) << 23);
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {
              if (c4 < ncb) {
                uint32_t r[32];
                ptx::tmem_ld_32x32(tmem + lane_addr + buf * OZ_BN + half * 128 + c4 * 32, r);
                ptx::tmem_ld_wait();
#pragma unroll
                for (int e = 0; e < 32; ++e)
                  S[c4 * 32 + e] = __fmaf_ru(__uint_as_float(r[e]), sc, S[c4 * 32 + e]);
              }
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&sm.tempty[buf]);
            if (++pc == nchunks) {
              pc = 0;
              ++pi;
            }
          }
          if (!ok) break;
          int32_t* pp = f.P + ((size_t)(kind == OZ_RAD_ADD ? args.slot_add : 0) * f.Np + gj0) *
                                  f.Mp + gi;
#pragma unroll
          for (int e = 0; e < 128; ++e) pp[(size_t)e * f.Mp] = __float_as_int(S[e]);
          continue;
        }
        if (kind == OZ_CRT && nchunks == 1) {
          // residue group (one modulus) of one chunk: the residue goes
          // straight from TMEM to res on the FP32 pipe, for the valid rows
          // and columns only (the reassembly reads no other); with several
          // chunks the int32 accumulation below is cheaper per chunk
          const int buf = acc & 1;
          const uint32_t par = (acc >> 1) & 1;
          ++acc;
          if (*(volatile int*)&sm.abort || !ptx::mbar_wait(&sm.tfull[buf], par, lim)) {
            if (!*(volatile int*)&sm.abort) raise_timeout(&sm, args.flag, 3);
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const float mf = (float)args.moduli[g];
          const float invf = __frcp_rn(mf);
          uint8_t* rp = f.res + (size_t)args.gres[g] * f.Np * f.Mp + (size_t)gj0 * f.Mp + gi;
          const size_t ld = (size_t)f.Mp;
          const int ncol = gi < f.M ? f.N - gj0 : 0;  // 0: a padding row
#pragma unroll 1
          for (int c8 = 0; c8 < 2; ++c8, rp += 64 * ld) {
            if (half * 2 + c8 >= f.nb) break;  // columns the tile did not multiply
            uint32_t r[64];  // two loads in flight per wait
            ptx::tmem_ld_32x32(tmem + lane_addr + buf * OZ_BN + half * 128 + c8 * 64, r);
            ptx::tmem_ld_32x32(tmem + lane_addr + buf * OZ_BN + half * 128 + c8 * 64 + 32, r + 32);
            ptx::tmem_ld_wait();
            // residue bytes: the residue rr < 256 is the low byte of the bits
            // of rr + 2^23.  Two columns per paired FP32 instruction: q and
            // r = RN(q (-m) + x), then 2^23 + r and 2^23 + m + r (both exact
            // integers below 2^24), the second kept where r < 0 (a float
            // compare, so that r = -0 keeps the first)
            const unsigned long long inv2 = f32x2(invf, invf), negm2 = f32x2(-mf, -mf),
                                     rnd2 = f32x2(12582912.0f, 12582912.0f),
                                     off2 = f32x2(8388608.0f, 8388608.0f),
                                     offm2 = f32x2(8388608.0f + mf, 8388608.0f + mf);
#pragma unroll
            for (int e = 0; e < 64; e += 2) {
              const unsigned long long x = f32x2(__uint_as_float(r[e]), __uint_as_float(r[e + 1]));
              const unsigned long long q = sub_x2(add_x2(mul_x2(x, inv2), rnd2), rnd2);
              const unsigned long long rr = fma_x2(q, negm2, x);
              const unsigned long long a = add_x2(rr, off2), b = add_x2(rr, offm2);
              r[e] = __uint_as_float((uint32_t)rr) < 0.0f ? (uint32_t)b : (uint32_t)a;
              r[e + 1] = __uint_as_float((uint32_t)(rr >> 32)) < 0.0f ? (uint32_t)(b >> 32)
                                                                      : (uint32_t)(a >> 32);
            }
            const int nc = ncol - c8 * 64;
            if (nc >= 64) {  // the common case: no per-column test
#pragma unroll
              for (int e = 0; e < 64; ++e) rp[e * ld] = (uint8_t)r[e];
            } else {
#pragma unroll
              for (int e = 0; e < 64; ++e)
                if (e < nc) rp[e * ld] = (uint8_t)r[e];
            }
          }
          ptx::tc_fence_before();
          __syncwarp();
          if (lane == 0) ptx::mbar_arrive(&sm.tempty[buf]);
          continue;
        }
        const int t = args.pl.gt[g];
        const int sh = 8 * (args.t_ref - t);
        const int npg = args.pl.gstart[g + 1] - args.pl.gstart[g];
        const int total = npg * nchunks;
        int c[128];
#pragma unroll
        for (int e = 0; e < 128; ++e) c[e] = 0;
        int cnt = 0;
        for (int idx = 0; idx < total; ++idx, ++acc) {
          const int buf = acc & 1;
          const uint32_t par = (acc >> 1) & 1;
          if (*(volatile int*)&sm.abort || !ptx::mbar_wait(&sm.tfull[buf], par, lim)) {
            if (!*(volatile int*)&sm.abort) raise_timeout(&sm, args.flag, 3);
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          // columns past N were not multiplied
          const int ncb = (f.nb * 64 - half * 128) >> 5;
#pragma unroll
          for (int c4 = 0; c4 < 4; ++c4) {
            if (c4 < ncb) {
              uint32_t r[32];
              ptx::tmem_ld_32x32(tmem + lane_addr + buf * OZ_BN + half * 128 + c4 * 32, r);
              ptx::tmem_ld_wait();
#pragma unroll
              for (int e = 0; e < 32; ++e) c[c4 * 32 + e] += __float2int_rn(__uint_as_float(r[e]));
            }
          }
          ptx::tc_fence_before();
          __syncwarp();
          if (lane == 0) ptx::mbar_arrive(&sm.tempty[buf]);
          ++cnt;
          const bool last_of_group = idx == total - 1;
          if ((cnt == OZ_FOLD_CHUNKS || last_of_group) && kind == OZ_CRT) {
            // CRT form: group g is modulus m_g; keep (A'B') mod m_g as a byte
            // in its residue plane [col][row], adding to an earlier fold of the group
            uint8_t* rp =
                f.res + (size_t)args.gres[g] * f.Np * f.Mp + (size_t)gj0 * f.Mp + gi;
            {
              const uint32_t m = (uint32_t)args.moduli[g];
              const uint32_t mg = 0xFFFFFFFFu / m;
              const bool first = cnt == idx + 1;  // no earlier fold in this group
#pragma unroll
              for (int e = 0; e < 128; ++e) {
                const int v = c[e];
                const uint32_t a = (uint32_t)(v < 0 ? -v : v);
                uint32_t r = a - __umulhi(a, mg) * m;
                if (r >= m) r -= m;
                if (r >= m) r -= m;
                if (v < 0 && r) r = m - r;
                if (!first) {
                  r += rp[(size_t)e * f.Mp];
                  if (r >= m) r -= m;
                }
                rp[(size_t)e * f.Mp] = (uint8_t)r;
                c[e] = 0;
              }
            }
            cnt = 0;
          } else if (cnt == OZ_FOLD_CHUNKS || last_of_group) {
            // fold into W (global, column-major, ld = Mp); the first fold of
            // a tile stores, later folds add
#pragma unroll
            for (int e = 0; e < 128; ++e) {
              long long* wp = args.W + (size_t)(gj0 + e) * args.Mp + gi;
              const long long v = shift_t(c[e], sh);
              *wp = have_w ? *wp + v : v;
              c[e] = 0;
            }
            have_w = true;
            cnt = 0;
          }
        }
      }
      if (!ok) break;
      if (args.mode != OZ_MID) continue;  // CRT residues / radius folds: combined later
      // ------------------------------------------------------ final epilogue
      const int Ei = (gi < args.M) ? args.Erow[(size_t)args.erow_stride * gi] : OZ_ZERO_EXP;
      double dlt = 0.0;
      if (args.mode == OZ_MID && gi < args.M) dlt = __dmul_ru((double)args.delta[gi], 0.515625);
      if (gi < args.M) {
        for (int e = 0; e < 128; ++e) {
          const int gj = gj0 + e;
          if (gj >= args.N) break;
          const long long v = args.W[(size_t)gj * args.Mp + gi];
          const int Fj = args.Fcol[(size_t)args.fcol_stride * gj];
          const bool zero = (Ei == OZ_ZERO_EXP) || (Fj == OZ_ZERO_EXP);
          const int ex = Ei + Fj - 8 * args.t_ref;
          double* Tp = args.T + (size_t)gj * args.Mp + gi;
          {
            double mlo = 0.0, mup = 0.0, tr = 0.0;
            if (!zero) {
              mlo = scale_dir(__ll2double_rd(v), ex, false);
              mup = scale_dir(__ll2double_ru(v + args.R), ex, true);
              const double bh = __dmul_ru(args.beta[gj], 0.5);
              const double x = __fma_ru(dlt, pow2_ru(Fj - 8), bh);
              tr = scale_dir(x, Ei - 8 * args.s, true);
            }
            const double err = __dadd_ru(tr, *Tp);
            double lo = __dsub_rd(mlo, err), up = __dadd_ru(mup, err);
            if (nonfinite) lo = up = __longlong_as_double(0x7ff8000000000000LL);
            double* cp = args.C + 2 * ((size_t)gi + (size_t)gj * args.ldc);
            cp[0] = lo;
            cp[1] = up;
          }
        }
      }
    }
  }

  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ------------------------------------------------------------- host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

int make_tmap(CUtensorMap* m, const void* base, int Kp, int rows, int planes, int box_rows,
              size_t pstride = 0) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return VCPCU_ERR_CUDA;
  }
  cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)Kp * 2,
                           (cuuint64_t)(pstride ? pstride : (size_t)Kp * rows) * 2};
  cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return VCPCU_ERR_CUDA;
  }
  return VCPCU_OK;
}

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

// The radius products and the residue GEMMs in one launch: the A planes are
// [residues (mpl) | |mA| + rA digits (sr) | rA digits (sr)] at one plane
// stride, the B planes [residues | rB digits | |mB| digits]; the groups of
// radius product 1, product 2 (each skipped for a point factor, point_mask
// as OzPlan's) and the moduli, each tagged with its kind.
void all_groups(const OzPairList& rad, const OzPairList& crt, int mpl, int sr, int point_mask,
                OzGemmArgs& a) {
  OzPairList& m = a.pl;
  int ng = 0, np = 0;
  auto add = [&](const OzPairList& src, int offA, int offB, int kind) {
    for (int g = 0; g < src.ngroups; ++g) {
      m.gstart[ng] = (int16_t)np;
      m.gt[ng] = src.gt[g];
      a.gkind[ng] = (int8_t)kind;
      a.gres[ng] = (int8_t)(kind == OZ_CRT ? g : 0);
      if (kind == OZ_CRT) a.moduli[ng] = OZ_MODULI[g];
      for (int q = src.gstart[g]; q < src.gstart[g + 1]; ++q, ++np) {
        m.pa[np] = (int8_t)(src.pa[q] + offA);
        m.pb[np] = (int8_t)(src.pb[q] + offB);
        m.pt[np] = src.pt[q];
      }
      ++ng;
    }
  };
  if (!(point_mask & 2)) add(rad, mpl, mpl, OZ_RAD_SET);
  if (!(point_mask & 1)) add(rad, mpl + sr, mpl + sr, OZ_RAD_ADD);
  add(crt, 0, 0, OZ_CRT);
  m.gstart[ng] = (int16_t)np;
  m.ngroups = ng;
  m.npairs = np;
}

}  // namespace

size_t oz_dyn_smem() { return (size_t)OZ_STAGES * STAGE_BYTES + 1024; }

// The dynamic shared-memory opt-in of the slice GEMM is a property of the
// device context: set it once per device ordinal (under a lock, since host
// threads may start products concurrently).
static int oz_gemm_smem_optin() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  VCPCU_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("slice GEMM: device ordinal %d out of range", dev);
    return VCPCU_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!done[dev]) {
    VCPCU_CUDA_TRY(cudaFuncSetAttribute(oz_slice_gemm_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)oz_dyn_smem()));
    done[dev] = true;
  }
  return VCPCU_OK;
}

int oz_run_gemm(const OzPlan& plan, int mode, const OzWorkspace& ws, double* C, long ldc,
                cudaStream_t st, int t_set) {
  const OzProblem& pb = plan.pb;
  if (int e = oz_gemm_smem_optin()) return e;
  OzGemmArgs a;
  memset(&a, 0, sizeof(a));
  int st_;
  const bool mid = mode == OZ_MID;
  const uint16_t* ap;
  const uint16_t* bp;
  int apl, bpl;
  if (mid) {
    ap = ws.a_mid; bp = ws.b_mid; apl = pb.mplanes; bpl = pb.mplanes;
    a.Erow = ws.E3 + 0; a.Fcol = ws.F2 + 0;
    a.pl = plan.mid; a.t_ref = plan.t_ref_mid; a.R = plan.R_mid;
  } else if (mode == OZ_RAD_SET) {  // (|mA| + rA) * rB
    ap = ws.a_p; bp = ws.b_r; apl = pb.sr; bpl = pb.sr;
    a.Erow = ws.E3 + 1; a.Fcol = ws.F2 + 1;
    a.pl = plan.rad; a.t_ref = plan.t_ref_rad; a.R = plan.R_rad;
  } else if (mode == OZ_RAD_ADD) {  // rA * |mB|
    ap = ws.a_r; bp = ws.b_s; apl = pb.sr; bpl = pb.sr;
    a.Erow = ws.E3 + 2; a.Fcol = ws.F2 + 0;
    a.pl = plan.rad; a.t_ref = plan.t_ref_rad; a.R = plan.R_rad;
  } else if (mode == OZ_ALL) {
    ap = ws.a_mid; bp = ws.b_mid;
    apl = bpl = pb.mplanes + 2 * pb.sr;
    a.Erow = ws.E3 + 0; a.Fcol = ws.F2 + 0;
    a.t_ref = plan.t_ref_rad; a.R = plan.R_rad;
    a.res = ws.res;
    all_groups(plan.rad, plan.crt, pb.mplanes, pb.sr, plan.point_mask, a);
  } else {  // OZ_CRT: residue products, one modulus per group
    ap = ws.a_mid; bp = ws.b_mid; apl = pb.L; bpl = pb.L;
    a.Erow = ws.E3 + 0; a.Fcol = ws.F2 + 0;
    a.pl = plan.crt; a.t_ref = 0; a.R = 0;
    a.res = ws.res;
    for (int l = 0; l < pb.L; ++l) a.moduli[l] = OZ_MODULI[l];
  }
  if (mode != OZ_ALL)
    for (int g = 0; g < a.pl.ngroups; ++g) {
      a.gkind[g] = (int8_t)mode;
      a.gres[g] = (int8_t)g;
    }
  if ((st_ = make_tmap(&a.tmA, ap, pb.Kp, pb.Mp, apl, OZ_BM, ws.a_pstride))) return st_;
  if ((st_ = make_tmap(&a.tmB, bp, pb.Kp, pb.Np, bpl, OZ_BN, ws.b_pstride))) return st_;
  a.M = pb.M; a.N = pb.N; a.Mp = pb.Mp; a.Np = pb.Np; a.Kp = pb.Kp;
  a.tiles_m = pb.Mp / OZ_BM;
  a.tiles_n = pb.Np / OZ_BN;
  a.mode = mode;
  a.t_set = t_set >= 0 ? t_set : (mode == OZ_RAD_SET ? 1 : 0);
  a.s = pb.s;
  a.erow_stride = 3;
  a.fcol_stride = 2;
  a.delta = ws.delta;
  a.beta = ws.beta;
  a.W = ws.W;
  a.T = ws.T;
  a.P = ws.P;
  a.slot_add = plan.rad_slots;
  a.C = C;
  a.ldc = ldc;
  a.flag = ws.flag;
  a.timeout_cycles = 4000000000LL;  // about 2 s at 2 GHz
  const int ntiles = a.tiles_m * a.tiles_n;
  const int nitems = mode == OZ_MID ? ntiles : ntiles * a.pl.ngroups;
  const int grid = nitems < num_sms() ? nitems : num_sms();
  oz_slice_gemm_kernel<<<grid, NTHREADS, oz_dyn_smem(), st>>>(a);
  VCPCU_LAUNCH_CHECK("oz_slice_gemm_kernel");
  return VCPCU_OK;
}

// One launch of the slice GEMM over all problems of a bucket: radius product
// 1 (OZ_RAD_SET), 2 (OZ_RAD_ADD) or the residue GEMMs (OZ_CRT).  `shape`
// supplies the pair lists (radius digit pairs, Lmax moduli), the fold count
// and the padded inner dimension shared by the bucket.
int oz_grun_gemm(const OzGBucket& b, const OzPlan& shape, int mode, int nitems, cudaStream_t st) {
  if (nitems <= 0) return VCPCU_OK;
  if (int e = oz_gemm_smem_optin()) return e;
  OzGemmArgs a;
  memset(&a, 0, sizeof(a));
  const size_t psA = (size_t)b.Mtot * b.Kp, psB = (size_t)b.Ntot * b.Kp;
  const uint16_t* ap;
  const uint16_t* bp;
  int apl, bpl;
  if (mode == OZ_RAD_SET) {  // (|mA| + rA) * rB
    ap = b.planesA + (size_t)b.Lmax * psA;
    bp = b.planesB + (size_t)b.Lmax * psB;
    apl = bpl = 2;
    a.pl = shape.rad;
    a.t_ref = shape.t_ref_rad;
  } else if (mode == OZ_RAD_ADD) {  // rA * |mB|
    ap = b.planesA + (size_t)(b.Lmax + 2) * psA;
    bp = b.planesB + (size_t)(b.Lmax + 2) * psB;
    apl = bpl = 2;
    a.pl = shape.rad;
    a.t_ref = shape.t_ref_rad;
  } else {
    ap = b.planesA;
    bp = b.planesB;
    apl = bpl = b.Lmax;
    a.pl = shape.crt;
    a.res = b.res;
    for (int l = 0; l < b.Lmax; ++l) a.moduli[l] = OZ_MODULI[l];
  }
  int st_;
  if ((st_ = make_tmap(&a.tmA, ap, b.Kp, b.Mtot, apl, OZ_BM))) return st_;
  if ((st_ = make_tmap(&a.tmB, bp, b.Kp, b.Ntot, bpl, 64))) return st_;
  a.bsub = 1;
  a.Kp = b.Kp;
  a.mode = mode;
  a.P = b.P;
  a.slot_add = shape.rad_slots;
  for (int g = 0; g < a.pl.ngroups; ++g) {
    a.gkind[g] = (int8_t)mode;
    a.gres[g] = (int8_t)g;
  }
  a.flag = b.flag;  // problem 0's status words take the (global) timeout bit
  a.timeout_cycles = 4000000000LL;  // about 2 s at 2 GHz
  a.gp = b.probs;
  a.gitem = mode == OZ_CRT ? b.item_crt : b.item_rad;
  a.gprob = mode == OZ_CRT ? b.prob_crt : b.prob_rad;
  a.gnprob = b.nprob;
  a.gnitems = nitems;
  const int grid = nitems < num_sms() ? nitems : num_sms();
  oz_slice_gemm_kernel<<<grid, NTHREADS, oz_dyn_smem(), st>>>(a);
  VCPCU_LAUNCH_CHECK("oz_slice_gemm_kernel");
  return VCPCU_OK;
}

}  // namespace vcpcu
