// ozaki.cuh -- Ozaki-scheme interval GEMM on tcgen05 tensor cores.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace vcpcu {

constexpr int OZ_MAX_SLICES = 12;
// Flag in a `slices` argument: radius products without their low x low
// digit pair, which the reassembly bounds (VCPCU_SLICES_FAST_RADIUS).
constexpr int OZ_FAST_RADIUS = 0x100;
// The slice count of a `slices` argument without the flag (0: default).
inline int oz_slice_count(int slices) { return slices & ~OZ_FAST_RADIUS; }
constexpr int OZ_MAX_RSLICES = 4;
constexpr int OZ_MAX_PAIRS = 80;
constexpr int OZ_MAX_GROUPS = 32;

// Tile geometry of the slice GEMM.
constexpr int OZ_BM = 128, OZ_BN = 256, OZ_BK = 64, OZ_STAGES = 4;

struct OzProblem {
  int M, N, K;     // logical sizes: C (M x N) = A (M x K) * B (K x N)
  int Mp, Np, Kp;  // padded: Mp % 128 == 0, Np % 256 == 0, Kp % 64 == 0
  int s, sr;       // digit slices of the midpoints / of the radius factors
  int crt;         // 1: midpoint by the CRT form (w-bit integers, L moduli)
  int w, L;        // CRT form: integer bits per operand, number of moduli
  int mplanes;     // midpoint planes per operand: s (slice form) or L (CRT form)
};

// Device scratch of one Ozaki-form product (pointers into one allocation).
struct OzWorkspace {
  uint16_t *a_mid, *a_p, *a_r;        // left digit planes  [s|sr][Mp][Kp] (bf16)
  uint16_t *b_mid, *b_r, *b_s;        // right digit planes [s|sr][Np][Kp] (bf16)
  unsigned long long* rowmax;         // [Mp][3] maxima of |mA|, P, rA (double bits)
  int* E3;                            // [Mp][3] exponents Em, Ep, Er
  unsigned long long* delta;          // [Mp] sum of |midpoint digits| per row
  int* F2;                            // [Np][2] exponents Fm, Fr
  double* beta;                       // [Np] sum_k |mB(k,j)| rounded up
  unsigned long long* asum;           // [Mp][4] CRT form: sum_k |A'(i,k)| as (bits >= 32, bits < 32);
                                      // sum_k lo^2 of the low radius digits of P, of rA
  uint8_t* res;                       // [L][Np][Mp] CRT form: residues of A'B' mod m_l
  double *midA, *radA;                // [K][M] midpoints / radii of A (column-major)
  double *midB, *radB;                // [Np][Kp] midpoints / radii of B (k contiguous)
  unsigned long long* bsum;           // [Np][4] CRT form: sum_k |B'(k,j)| as (bits >= 32, bits < 32);
                                      // sum_k lo^2 of the low radius digits of rB, of |mB|
  double* T;                          // [N][Mp] upper bound of the radius product (slice form)
  long long* W;                       // [Np][Mp] int64 fold buffer (slice form)
  int32_t* P;                         // [2 slots][Np][Mp] fp32 folds (bits) of the two radius products
  int* flag;                          // [0] non-finite input, [1] device wait timeout
  // Plane strides (elements) of the left / right digit planes when they are
  // a row / column block of larger planes; 0: Mp Kp / Np Kp.
  size_t a_pstride = 0, b_pstride = 0;
};

// Ordered list of slice pairs grouped by t = p + q (1-based slice numbers).
struct OzPairList {
  int npairs, ngroups;
  int8_t pa[OZ_MAX_PAIRS], pb[OZ_MAX_PAIRS];   // 0-based plane indices
  int8_t pt[OZ_MAX_PAIRS];                     // t = p + q of pair (1-based digits)
  int16_t gstart[OZ_MAX_GROUPS + 1];           // group g = pairs [gstart[g], gstart[g+1])
  int8_t gt[OZ_MAX_GROUPS];                    // t of group g (radius list: the largest)
};

// OZ_RAD_SET: radius product 1, (|mA| + rA) * rB; OZ_RAD_ADD: radius
// product 2, rA * |mB|.  Each writes T or adds to it (OzGemmArgs::t_set).

enum OzMode { OZ_RAD_SET = 0, OZ_RAD_ADD = 1, OZ_MID = 2, OZ_CRT = 3, OZ_ALL = 4 };
// OZ_ALL (CRT form): both radius products and the residue GEMMs in one
// launch -- one pair list over all planes, the mode of each group in
// OzGemmArgs::gkind (fewer launch tails, most of all for the blocks of the
// host-pointer pipeline).

struct alignas(128) OzGemmArgs {
  CUtensorMap tmA;  // left digit planes, dims {Kp, Mp, planes}
  CUtensorMap tmB;  // right digit planes, dims {Kp, Np, planes}
  int M, N, Mp, Np, Kp;
  int tiles_m, tiles_n;
  int t_ref, R;     // W unit 2^(E_i + F_j - 8 t_ref); R = floor-shifted folds
  int mode;
  int t_set;        // radius modes: 1 T = product, 0 T +=RU product
  int s;            // midpoint slices (OZ_MID truncation bound)
  const int* Erow;  // row exponent of the left operand:  Erow[erow_stride * i]
  int erow_stride;
  const int* Fcol;  // column exponent of the right operand: Fcol[fcol_stride * j]
  int fcol_stride;
  const unsigned long long* delta;
  const double* beta;
  long long* W;
  double* T;
  double* C;        // interval output (kv layout), OZ_MID
  long ldc;
  int* flag;
  long long timeout_cycles;
  uint8_t* res;                 // OZ_CRT: residue planes [L][Np][Mp]
  int moduli[32];               // OZ_CRT: modulus of group g
  int32_t* P;                   // radius groups: the fold of a tile -> slot 0 (product 1) or
  int slot_add;                 //   slot slot_add (product 2, OZ_RAD_ADD)
  int8_t gkind[OZ_MAX_GROUPS];  // mode of group g (OZ_RAD_SET / _ADD / OZ_CRT / OZ_MID)
  int8_t gres[OZ_MAX_GROUPS];   // OZ_CRT groups: residue plane (modulus index) of group g
  // grouped products: items of problem p are [gitem[p], gitem[p+1]); its
  // tiles read rows gp[p].rowoff.. / gp[p].coloff.. of the stacked planes and
  // write res + gp[p].res_off / P + gp[p].P_off (null gp: one product)
  const struct OzGProb* gp;
  const int* gitem;
  const int* gprob;  // item -> problem (one load per item)
  int gnprob, gnitems;
  // bsub != 0 (grouped products): tmB has 64-row boxes and a tile loads and
  // multiplies only the 64-column blocks that hold columns of its problem
  // (MMA N = 64, 128, 192 or 256); else one 256-row box, N = 256
  int bsub;
  OzPairList pl;
};

// Plan of one product (host side): slice counts, the pair lists and the
// W scaling, shared with the host model.
struct OzPlan {
  OzProblem pb;
  OzPairList mid, rad, crt;
  int t_ref_mid, R_mid, t_ref_rad, R_rad;
  uint32_t Q[16][4];   // CRT basis: Q_l = (M/m_l) * ((M/m_l)^-1 mod m_l), 32-bit limbs
  uint32_t Mlimb[4];   // M = prod m_l
  // bit 0: A is a point matrix (rA = 0), bit 1: B is (rB = 0).  The radius
  // product with a zero factor is skipped; it would add exactly 0 to T.
  int point_mask = 0;
  // Folds of one radius product: one fp32 upper bound per (product, tile),
  // the epilogue's weighted upward sum of all its digit pairs (rad_slots = 1).
  int rad_slots;
  // 1: the radius products leave out the pair of the two low digits (CRT
  // form with OZ_FAST_RADIUS); the reassembly adds its bound.
  int rad_lowb;
};

// The radius bound T(i, j) from the folds of the two radius products (the
// same values the radius epilogue would write): passed by value to kernels.
struct OzRadConst {
  int nslot;                    // folds per product (slots [0, n) and [n, 2n))
  int run1, run2;               // which products ran (zero-radius operands skip)
  int t_ref, R;
  int lowb;                     // 1: the pair of the two low digits was left out of
                                // both products; T adds its Cauchy-Schwarz bound
};
OzRadConst oz_rad_const(const OzPlan& plan);
// Slice form: T from the folds into ws.T (the CRT form's reassembly
// computes it in place).
int oz_radius_T(const OzPlan& plan, const OzWorkspace& ws, cudaStream_t st);

// crt != 0 selects the CRT form of the midpoint with w = 7 * s integer bits.
// s may carry OZ_FAST_RADIUS (CRT form: the radius products leave out
// their low x low digit pair) and is then 0 for the default 8.
int oz_make_plan(int M, int N, int K, int s, int sr, OzPlan* plan, int crt = 0);
int oz_crt_assemble(const OzPlan& plan, const OzWorkspace& ws, double* C, long ldc,
                    cudaStream_t st);
int oz_prepare(const OzProblem& pb, const double* A, long lda, const double* B, long ldb,
               OzWorkspace& ws, cudaStream_t st);
// oz_prepare in parts: clear the row maxima, sums and status words; midrad
// and row maxima of the columns [k0, k1) of A (any order of column ranges,
// the maxima accumulate); row exponents and the left planes; the right
// planes (CRT form) of B, whose columns may be any column panel of a larger
// right factor.
int oz_prepare_left_begin(const OzProblem& pb, OzWorkspace& ws, cudaStream_t st);
int oz_prepare_left_rowmax(const OzProblem& pb, const double* A, long lda, int k0, int k1,
                           OzWorkspace& ws, cudaStream_t st);
int oz_prepare_left_finish(const OzProblem& pb, OzWorkspace& ws, cudaStream_t st);
int oz_prepare_right_crt(const OzProblem& pb, const double* B, long ldb, OzWorkspace& ws,
                         cudaStream_t st, int colbase = 0, int cols = -1, size_t pstride = 0);
// Left planes of the row block [i0, i0 + rows) (i0 and rows multiples of
// 128, padding rows included) from the rows of A alone: midrad, row maxima,
// exponents and planes (CRT form), after oz_prepare_left_begin.  B's column
// blocks: oz_prepare_right_crt with colbase = j0 and cols its padded width
// (B points at column 0; planes, F2 and beta of the whole right factor).
int oz_prepare_left_rows(const OzProblem& pb, const double* A, long lda, int i0, int rows,
                         OzWorkspace& ws, cudaStream_t st);
// t_set < 0: the radius product of OZ_RAD_SET writes T, that of OZ_RAD_ADD
// adds to it; 0 / 1 force add / write.
int oz_run_gemm(const OzPlan& plan, int mode, const OzWorkspace& ws, double* C, long ldc,
                cudaStream_t st, int t_set = -1);
size_t oz_workspace_bytes(const OzProblem& pb);
int oz_carve_workspace(const OzProblem& pb, void* base, OzWorkspace* ws);

// Read and clear the sticky status (bit 0 non-finite input, bit 1 timeout);
// synchronises the stream.
int oz_take_status(cudaStream_t s, int* status);
// A bounded wait on an mbarrier nothing arrives on: sets the timeout status.
int oz_selftest_timeout(long long limit, cudaStream_t s);
// Merge a product's status words into the sticky device status.
void oz_merge_status(const int* flag, cudaStream_t s);
// Device address of the sticky status word of the current device (kernels
// that merge statuses themselves atomicOr into it); null on error.
int* oz_status_ptr();

// dd GEMM (pddblas semantics) by the CRT form: C, Cerr as documented in
// include/vcpcuda.h.  static_scratch != nullptr: use that device buffer of
// static_bytes instead of allocating.
int ozaki_ddgemm(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                 double* C, long ldc, double* Cerr, long lde, int slices, cudaStream_t s,
                 void* static_scratch = nullptr, size_t static_bytes = 0);
int dd_plan_bits(int k, int slices, int* w, int* L);

// Per-phase timing of the Ozaki form (0 prep, 1 radius 1, 2 radius 2,
// 3 midpoint / residue GEMMs, 4 reassembly): CUDA events on the call's
// stream while profiling is enabled.
int oz_profile_enable(int on);
int oz_profile_read(double* ms, int nphases, long long* flops);
struct PhaseTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  int phase;
  cudaStream_t s;
  PhaseTimer(int ph, cudaStream_t st);
  ~PhaseTimer();
};
void oz_profile_add_flops(long long f);

// Operand preparation, the three slice-GEMM phases and the reassembly of
// one planned product (shared by every entry point of the Ozaki form).
int oz_run_product(const OzPlan& plan, OzWorkspace& ws, const double* A, long lda,
                   const double* B, long ldb, double* C, long ldc, cudaStream_t s);

// ---------------------------------------------------------------------------
// Grouped CRT-form products (a batch of uneven interval products in a few
// launches).  Problems with the same padded inner dimension Kp, modulus
// count and operand width form a bucket (cut into chunks of similar work);
// the bucket's operand planes are stacked: the rows of problem p occupy rows
// [rowoff, rowoff + Mp) of the A planes ([plane][Mtot][Kp]) and [coloff,
// coloff + Np) of the B planes ([plane][Ntot][Kp]); its residue bytes and
// radius folds live at res_off / P_off of the bucket's arrays, laid out as
// in a single product.  Every kernel of the CRT form has a grouped twin
// that finds its problem by a binary search over a prefix array of blocks,
// or by one load from a block / item -> problem table.
struct OzGProb {
  int m, n, k;
  const double* A;
  long lda;
  const double* B;
  long ldb;
  double* C;
  long ldc;
  int Mp, Np, L, w;
  int rowoff, coloff;          // stacked rows of the bucket's A / B planes
  int tiles_m, tiles_n;
  long long res_off, P_off;    // element offsets into the bucket's res / P
  int orig;                    // index in the caller's problem table
  uint32_t Q[16][4];           // CRT basis of this problem's L moduli
  uint32_t Mlimb[4];
  float invMf;                 // 2^64 / M rounded to float
};

// Device view of one bucket (all pointers device memory).
struct OzGBucket {
  int nprob, Kp, Lmax, Mtot, Ntot;
  const OzGProb* probs;
  const int* blk_rowmax;   // [nprob + 1] prefix of rowmax blocks
  const int* blk_split;    // [nprob + 1] prefix of split_left blocks
  const int* item_rad;     // [nprob + 1] prefix of radius work items (groups x tiles)
  const int* item_crt;     // [nprob + 1] prefix of residue work items (L x tiles)
  const int* prob_rad;     // [radius items] the problem of each item
  const int* prob_crt;     // [residue items] the problem of each item
  const int* blk_asm;      // [nprob + 1] prefix of reassembly blocks
  const int* prob_asm;     // [reassembly blocks] the problem of each block
  const int* col_prob;     // [Ntot] problem of each stacked B column
  uint16_t* planesA;       // [Lmax + 4][Mtot][Kp]: residues, |mA|+rA digits, rA digits
  uint16_t* planesB;       // [Lmax + 4][Ntot][Kp]: residues, rB digits, |mB| digits
  unsigned long long* rowmax;  // [Mtot][3]
  int* E3;                 // [Mtot][3]
  int* F2;                 // [Ntot][2]
  double* beta;            // [Ntot]
  double *midB, *radB;     // [Ntot][Kp] midrad of the stacked B columns
  double *midA, *radA;     // [Kp][Mtot] midrad of the stacked A rows (column-major)
  unsigned long long* bsum;  // [Ntot][4] as OzWorkspace::bsum
  unsigned long long* asum;  // [Mtot][4] as OzWorkspace::asum
  uint8_t* res;
  int32_t* P;
  int* flag;               // [nprob][4]: non-finite input, wait timeout
  unsigned long long* t_first;  // per caller problem (may be null)
  unsigned long long* t_last;
};

// Kernels of the grouped form (ozaki_split.cu, ozaki_gemm.cu, ozaki_crt.cu).
// wmax: the largest operand width w of the bucket (selects the limb form)
int oz_gprep(const OzGBucket& b, int nblk_rowmax, int nblk_split, int wmax, cudaStream_t st);
int oz_grun_gemm(const OzGBucket& b, const OzPlan& shape, int mode, int nitems,
                 cudaStream_t st);
// shape: the bucket's plan (every problem of a bucket has the same CRT basis)
int oz_gassemble(const OzGBucket& b, const OzPlan& shape, const OzRadConst& rc, int nblk,
                 cudaStream_t st);
// The grouped CRT-form product of a batch (batch.cu's tensor-core path).
// oz_group_plan builds the buckets and uploads their tables (outside any
// stream capture); oz_group_record launches the kernels of every bucket on
// one stream (capturable); oz_group_free releases the plan.  With
// persistent != 0 the device memory comes from cudaMalloc (kept for graph
// replays), else from the stream-ordered allocator of `s`.
struct BatchProblemView {
  int m, n, k, lda, ldb, ldc;
  const double* A;
  const double* B;
  double* C;
};
struct OzGroupPlan;
int oz_group_plan(int count, const BatchProblemView* problems, const char* select, int slices,
                  int persistent, cudaStream_t s, OzGroupPlan** out);
int oz_group_record(OzGroupPlan* g, unsigned long long* t_first, unsigned long long* t_last,
                    cudaStream_t s);
void oz_group_free(OzGroupPlan* g, cudaStream_t s);

// CRT-form product of host matrices (column-major, lda = m, ldb = k,
// ldc = m) with the host<->device copies overlapped: C is cut into
// row_panels x panels blocks; A goes up in row blocks and B in column
// blocks, interleaved, and each block of C is multiplied, reassembled and
// sent down as soon as its row block of A and column block of B are on the
// device and prepared.  Streams: `s` prepares the operand blocks, the block
// products alternate between `c0` and `c1` (each with its own residue and
// fold buffers), `up` / `down` copy.  Bit-identical to ozaki_igemm on the
// same operands (every entry depends on its row of A and column of B only).
// Synchronises before returning.
int ozaki_igemm_host_pipelined(int m, int n, int k, const double* A, const double* B, double* C,
                               int slices, int panels, int row_panels, cudaStream_t s,
                               cudaStream_t c0, cudaStream_t c1, cudaStream_t up,
                               cudaStream_t down);

// point_mask as OzPlan::point_mask (the caller guarantees the zero radii).
int ozaki_igemm(int m, int n, int k, const double* A, long lda, const double* B, long ldb,
                double* C, long ldc, int form, int slices, cudaStream_t s, int point_mask = 0);

}  // namespace vcpcu
