/*
 * vcpcuda.h -- C ABI of the GB300 (sm_103a) verified dense matrix product.
 *
 * Every function returns an int status (VCPCU_OK == 0).  No C++ exception and
 * no CUDA/torch type crosses this boundary: pointers are plain `double*`,
 * streams are passed as `void*` (a cudaStream_t, NULL = legacy default stream).
 * Matrices are column-major, as in vcp::mats<T> (vcp/mats.hpp:411-417).
 * Intervals are stored like kv::interval<double>: two doubles {inf, sup}
 * per entry, 16 bytes, so a std::vector<kv::interval<double>> can be passed
 * as `const double*` with no repacking.
 *
 * The library never touches the caller's host floating-point rounding mode:
 * every directed rounding happens per instruction on the GPU.
 *
 * Two kinds of entry points:
 *   - "host" entry points keep the reference signatures (vblas rmatmul /
 *     udmatmul) and take host pointers; they copy to the device, run, copy
 *     back and synchronise.  They are the drop-in replacement.
 *   - "_dev" entry points take device pointers and leading dimensions and
 *     are ordered on the given stream (asynchronous w.r.t. the host).
 */
#ifndef VCPCUDA_H
#define VCPCUDA_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define VCPCU_OK               0
#define VCPCU_ERR_INVALID_ARG  1  /* bad shape, leading dimension, pointer or flag   */
#define VCPCU_ERR_CUDA         2  /* a CUDA runtime/driver call failed               */
#define VCPCU_ERR_NONFINITE    3  /* Ozaki form: an input entry is Inf or NaN        */
#define VCPCU_ERR_RANGE        4  /* Ozaki form: exponent outside the split range    */
#define VCPCU_ERR_TIMEOUT      5  /* a bounded device-side wait gave up              */
#define VCPCU_ERR_UNSUPPORTED  6  /* no usable sm_103 device, or option not built    */
#define VCPCU_ERR_ALLOC        7  /* device or pinned host allocation failed         */
#define VCPCU_ERR_VERIFY       8  /* a verification condition failed (||RA - I|| >= 1) */
#define VCPCU_ERR_IO           9  /* a .vcpmat file could not be read or written       */

/* rounding_mode values, identical to vblas rmatmul (vblas/rmatmul.hpp:100-102) */
#define VCPCU_ROUND_UP      1
#define VCPCU_ROUND_NEAREST 0
#define VCPCU_ROUND_DOWN   -1

/* interval-product forms */
#define VCPCU_FORM_PLAIN 0   /* FP64 CUDA cores, __fma_rd/__fma_ru, pidblas order   */
#define VCPCU_FORM_OZAKI 1   /* error-free bf16 slices on tcgen05 tensor cores       */
#define VCPCU_FORM_AUTO  2   /* autotuned choice of form and slice count            */
#define VCPCU_FORM_OZAKI_SLICES 3 /* tensor cores, midpoint by triangular slice pairs */

/* Added to `slices` of VCPCU_FORM_OZAKI (0x100 + s, or 0x100 alone for the
 * default s): the two radius products leave out the pair of the two low
 * digits of their 2-digit factors and add its Cauchy-Schwarz bound instead
 * (6 bf16 GEMMs instead of 8; the default runs all four pairs).  It costs
 * about 4e-5 of the enclosure width where the magnitudes of a row / column
 * of the radius factors lie within one binade, 4e-4 where they spread over
 * 2^16 and up to 3 % over 2^64, and up to a fifth of the radius term where
 * most entries lie some 2^7 below their row's largest (R [A] with A near
 * the identity): FORM_AUTO takes it where a probe finds it no wider than
 * the plain form. */
#define VCPCU_SLICES_FAST_RADIUS 0x100

/* ---- diagnostics ----------------------------------------------------------- */

/* Text of the last error raised on the calling host thread ("" if none). */
const char* vcpcu_last_error_string(void);

/* Library version as an integer (major*10000 + minor*100 + patch). */
int vcpcu_version(void);

/* Number of kernels this library launched since load (all threads). */
long long vcpcu_launch_count(void);

/* Synchronise `stream` and report (then clear) the sticky device status of
 * earlier stream-ordered Ozaki-form calls on the current device:
 * VCPCU_ERR_NONFINITE if one saw an Inf/NaN input (its output is NaN),
 * VCPCU_ERR_TIMEOUT if a bounded device-side wait gave up (its output is
 * invalid), else VCPCU_OK.  The host-pointer entry points check this
 * themselves. */
int vcpcu_status(void* stream);

/* Self-test of that timeout path: one thread waits, with the same bounded
 * mbarrier wait as the tensor-core kernels, on a barrier that nothing ever
 * arrives on; after limit_cycles (0: 2e9, about 1 s) it gives up, sets the
 * timeout status and returns, and the call returns what vcpcu_status then
 * reports: VCPCU_ERR_TIMEOUT when the path works.  No fault, trap or hang;
 * the context stays usable. */
int vcpcu_selftest_timeout(long long limit_cycles, void* stream);

/* Per-phase timing of Ozaki-form calls: while enabled, every call records
 * CUDA events on its own stream around its phases (0 operand preparation,
 * 1 and 2 the two radius slice GEMMs, 3 the midpoint slice GEMM, 4 the
 * reassembly of the CRT form).  vcpcu_profile_read waits for the recorded events, writes
 * the summed milliseconds of the first `nphases` phases to ms[], the summed
 * algorithmic tensor-core flops (2 m n k per slice pair) to *tensor_flops,
 * and clears the record.  No counterpart in the reference (it has only
 * vcp::time tic/toc, vcp/vcp_timer.hpp:39-62). */
int vcpcu_profile(int enable);
int vcpcu_profile_read(double* ms, int nphases, long long* tensor_flops);

/* ---- directed-rounding point GEMM ----------------------------------------- */

/* Replaces vblas rmatmul (vblas/rmatmul.hpp:102):
 *   void rmatmul(int m, int n, int k, const double* A, const double* B,
 *                double* C, int rounding_mode);
 * A is m x n, B is n x k, C is m x k (inner dimension n, the vblas naming).
 * Every C entry is the sequential FMA chain over the inner index in
 * ascending order, each FMA rounded in `rounding_mode` (1 up, -1 down,
 * anything else nearest), starting from +0.0 -- the result definition of
 * vblas (vblas/README.md, "packing layout").  m <= 0 or k <= 0: no-op;
 * n <= 0: C is zeroed (vblas/rmatmul_avx512.hpp:482-490).  Host pointers;
 * synchronous. */
int vcpcu_rmatmul(int m, int n, int k, const double* A, const double* B,
                  double* C, int rounding_mode);

/* Replaces vblas udmatmul (vblas/udmatmul.hpp:758): CU = fl_up(A*B) and
 * CD = fl_down(A*B) in one pass, same shapes and chain definition as
 * vcpcu_rmatmul.  Host pointers; synchronous. */
int vcpcu_udmatmul(int m, int n, int k, const double* A, const double* B,
                   double* CU, double* CD);

/* Device-pointer, stream-ordered forms of the two calls above, with
 * leading dimensions (lda >= m, ldb >= n, ldc >= m). */
int vcpcu_rmatmul_dev(int m, int n, int k, const double* A, int lda,
                      const double* B, int ldb, double* C, int ldc,
                      int rounding_mode, void* stream);
int vcpcu_udmatmul_dev(int m, int n, int k, const double* A, int lda,
                       const double* B, int ldb, double* CU, double* CD,
                       int ldc, void* stream);

/* Tensor-core enclosure of a point product in the shape of vblas udmatmul
 * (vblas/udmatmul.hpp:758): CD <= A*B <= CU entrywise, rigorous, but not
 * the FMA-chain bits of vcpcu_udmatmul.  A is m x n, B is n x k, C is
 * m x k (vblas naming).  The product is the Ozaki form of vcpcu_igemm_dev
 * on zero-radius operands with the radius products skipped: residues of
 * w = 7 * slices bit scaled integers (0 = default 8), Chinese remaindering,
 * truncation bound.  m <= 0 or k <= 0: no-op; n <= 0: CU = CD = 0.
 * Requires finite inputs (VCPCU_ERR_NONFINITE).  The _dev form is
 * stream-ordered (status through vcpcu_status); the host form is
 * synchronous. */
int vcpcu_udmatmul_ozaki_dev(int m, int n, int k, const double* A, int lda,
                             const double* B, int ldb, double* CU, double* CD,
                             int ldc, int slices, void* stream);
int vcpcu_udmatmul_ozaki(int m, int n, int k, const double* A, const double* B,
                         double* CU, double* CD, int slices);

/* ---- interval GEMM (pidblas::mulmm, vcp/pidblas.hpp:239-294) -------------- */

/* C = [A] * [B] for interval matrices in kv layout ({inf,sup} pairs).
 * BLAS naming: A is m x k (lda >= m, in interval entries), B is k x n,
 * C is m x n.  The result encloses every exact product of point matrices
 * taken from [A] and [B].
 *   form == VCPCU_FORM_PLAIN: bit-identical to pidblas::mulmm over a dgemm
 *     whose every entry is the ascending sequential FMA chain (vblas
 *     rmatmul): lC = RD(mA*mB), uC = RU(mA*mB), T = RU((|mA|+rA)*rB) +RU
 *     RU(rA*|mB|), uC +=RU T, lC -=RD T.  `slices` is ignored.
 *   form == VCPCU_FORM_OZAKI: tensor-core form.  The midpoints are scaled
 *     per row / column to w = 7 * slices bit integers (2 <= slices <= 12;
 *     0 = default 8, w = 56); their product is exact, from residues modulo
 *     up to 16 moduli <= 256 (one bf16 GEMM each, Chinese remaindering);
 *     the rounding of the midpoints to w bits, the radius term (upward bf16
 *     digit slices, see VCPCU_SLICES_FAST_RADIUS) and the final roundings
 *     are bounded upward.  Requires
 *     finite inputs (NaN results and VCPCU_ERR_NONFINITE otherwise) and
 *     16-byte aligned A and B.
 *   form == VCPCU_FORM_OZAKI_SLICES: as OZAKI, but the midpoint product is
 *     the triangular sum of `slices` balanced 8-bit digit slices per operand
 *     (the classic Ozaki splitting) with a rigorous truncation bound.
 *   form == VCPCU_FORM_AUTO: the autotuner picks the form and slice count.
 * Device pointers; stream-ordered; scratch comes from the stream-ordered
 * allocator of the current device. */
int vcpcu_igemm_dev(int m, int n, int k, const double* A, int lda,
                    const double* B, int ldb, double* C, int ldc,
                    int form, int slices, void* stream);

/* Host-pointer, synchronous form of vcpcu_igemm_dev (lda = m, ldb = k,
 * ldc = m): the drop-in for a std::vector<kv::interval<double>> product.
 * When the tensor-core CRT form runs (form OZAKI, or AUTO choosing it) and
 * n >= 2048, the copies overlap the computation: C is cut into blocks (row
 * blocks of about 1365 rows, at most 6, and column blocks of 1024 columns,
 * at most 4;
 * the environment variables VCPCU_HOST_ROW_PANELS and VCPCU_HOST_PANELS
 * override the counts, 1 and 1 turn the overlap off), A goes to the device in
 * row blocks and B in column blocks, interleaved, each block of C is
 * prepared, multiplied and reassembled as soon as its operands have landed,
 * and it comes back while the next block computes.  The result is
 * bit-identical to one vcpcu_igemm_dev call.  Pinned (page-locked) host
 * buffers let the copies run asynchronously. */
int vcpcu_igemm(int m, int n, int k, const double* A, const double* B,
                double* C, int form, int slices);

/* ---- interval x point, [A]^T[A], verified A^T A, ||R[A] - I|| ------------ */

/* Mixed interval / point products, GEMM naming (L m x k, R k x n, C m x n):
 *   interval_side == 0: C = [L] * R, L interval, R point -- replaces
 *     pidblas::mul_im_m (vcp/pidblas.hpp:90-140);
 *   interval_side == 1: C = L * [R], L point, R interval -- replaces
 *     pidblas::mul_m_im (vcp/pidblas.hpp:142-196).
 * Point matrices are plain doubles, intervals kv pairs.  The plain form is
 * bit-identical to pidblas over a sequential-chain dgemm (lC = RD(mid*P),
 * uC = RU(mid*P), temp = RU(rad*|P|), uC +=RU temp, lC -=RD temp); the
 * Ozaki forms enclose the same product. */
int vcpcu_igemm_point_dev(int interval_side, int m, int n, int k,
                          const double* L, int ldl, const double* R, int ldr,
                          double* C, int ldc, int form, int slices, void* stream);
int vcpcu_igemm_point(int interval_side, int m, int n, int k, const double* L,
                      const double* R, double* C, int form, int slices);

/* C (n x n) = [A]^T [A] for an interval A (k x n) -- replaces
 * pidblas::mulltmm (vcp/pidblas.hpp:296-358; matrix::ltransmul,
 * vcp/matrix.hpp:405-415).  Plain form: bit-identical to pidblas over
 * sequential-chain dsyrk/dgemm (upper triangle computed, mirrored). */
int vcpcu_isyrk_dev(int n, int k, const double* A, int lda, double* C, int ldc,
                    int form, int slices, void* stream);
int vcpcu_isyrk(int n, int k, const double* A, double* C, int form, int slices);

/* C (n x n, intervals) = [RD(A^T A), RU(A^T A)] for a point A (k x n), each
 * entry the sequential chain -- replaces pidblas::vmulmm
 * (vcp/pidblas.hpp:198-236). */
int vcpcu_vsyrk_dev(int n, int k, const double* A, int lda, double* C, int ldc,
                    void* stream);
int vcpcu_vsyrk(int n, int k, const double* A, double* C);

/* Upper bound of ||R [A] - I||_inf for a point R and an interval A (n x n):
 * the check of imats::linearsolve (vcp/imats.hpp:316-336; mats::norminf,
 * vcp/mats.hpp:1583-1597): RA by vcpcu_igemm_point (side 1) in `form`,
 * the diagonal shifted by -1 outward, per row the upward sum of |.| in
 * ascending column order, then the largest row sum.  The _dev form writes
 * the bound to device memory (*bound), the host form to host memory. */
int vcpcu_norm_I_minus_RA_dev(int n, const double* R, int ldr, const double* A,
                              int lda, double* bound, int form, int slices,
                              void* stream);
int vcpcu_norm_I_minus_RA(int n, const double* R, const double* A, double* bound,
                          int form, int slices);

/* The verification of imats::linearsolve (vcp/imats.hpp:293-364) once its
 * approximate inverse R = inv(mid [A]) and approximate solution
 * mx = R mid([b]) are formed (the reference forms both on the host: LAPACK
 * inverse, BLAS product, :299-302).  A is n x n interval, b and x n x nrhs
 * interval, R n x n point, mx n x nrhs point, all column-major (kv layout
 * for intervals).  Steps, each with the reference's kv arithmetic:
 *   P = [A] mx - [b];  r = R P;  E = R [A] - I;  G = ||E||_inf (upper);
 *   t = || |r| ||_inf;  g = [t, t] / (1 - [G, G]);
 *   H = |E| (g ... g);  x = mx + [-u, u] with u = sup|r| + sup H (upward).
 * R[A] runs in `form`; the three products with nrhs columns run in the
 * plain form when nrhs <= 4 (a thin FP64 kernel), else in `form` too.  In
 * the plain form every bit of x and G equals the reference's (for n >= 2:
 * with n = 1 the reference takes its scalar shortcuts).  *bound receives G;
 * the reference throws vcp::verification_error when G >= 1 (x is then
 * meaningless): the host form returns VCPCU_ERR_VERIFY in that case, the
 * _dev form leaves the test to the caller (*bound in device memory).
 * Inputs must be finite. */
int vcpcu_ilss_verify_dev(int n, int nrhs, const double* A, int lda, const double* b, int ldb,
                          const double* R, int ldr, const double* mx, int ldmx, double* x,
                          int ldx, double* bound, int form, int slices, void* stream);
int vcpcu_ilss_verify(int n, int nrhs, const double* A, const double* b, const double* R,
                      const double* mx, double* x, double* bound, int form, int slices);

/* ---- Legendre generator: tensor-product basis matrices --------------------- */

/* Replaces the element loops that build the two-dimensional Legendre basis
 * at the Gauss-Legendre points, Legendre_Bases_Generator::phi_point_set
 * (vcp/ldbase.hpp:355-374), and the weight * uh^p scaling inside
 * uhphiphi's element loop (vcp/ldbase.hpp:994-1001), so that uhphiphi
 * becomes the interval product Phi diag(w uh^p) Phi^T.  Writes the n x P
 * interval matrix (kv layout; P = nqa * nqb)
 *   out(i, q) = Ta(ia[i], qa) * Tb(ib[i], qb) [* s1(q)] [* s2(q)],
 *   q = qa * nqb + qb (the reference's Pointlist order),
 * at out + 2 (i + q ld), or at out + 2 (q + i ld) when transposed (P x n).
 * Ta, Tb: nt x nqa and nt x nqb interval tables (one-dimensional basis
 * values, row = basis index), column-major; ia, ib: nb device ints in
 * [0, nt) (an index outside gives a NaN entry); s1, s2: optional interval
 * vectors of length P (NULL to skip).  Every factor is an interval product
 * with directed rounding; accumulate adds the result to the entry already
 * in out (round down / up).  All pointers are device pointers; interval
 * arrays 16-byte aligned. */
int vcpcu_tensor_basis_dev(int nb, const int* ia, const int* ib, int nt, const double* Ta,
                           const double* Tb, int nqa, int nqb, const double* s1,
                           const double* s2, double* out, long ld, int transposed,
                           int accumulate, void* stream);

/* ---- inf-sup interval FMA (vcp/ifma.hpp, vcp/pidblas_fma.hpp) ------------- */

/* Replaces vcp::ifma (vcp/ifma.hpp:48-139), elementwise over kv pairs:
 *   R[i] = ifma(A[i], B[i], C[i]) encloses {x y + z : x in A[i], y in B[i],
 *   z in C[i]}, with the sign-case selection and directed fused
 *   multiply-adds of the reference's portable branch (bit-identical).
 * R may alias C.  Finite inputs.  A, B 16-byte aligned (_dev form). */
int vcpcu_ifma_dev(long count, const double* A, const double* B, const double* C,
                   double* R, void* stream);
int vcpcu_ifma(long count, const double* A, const double* B, const double* C,
               double* R);

/* Replaces vcp::pidblas_fma::mulmm (vcp/pidblas_fma.hpp:46-80):
 * C = [A] [B] (kv layout, A m x k, B k x n, C m x n) with every entry the
 * ifma chain over the inner index in ascending order from [0, 0] --
 * bit-identical to the reference loop; FP64 pipe (2 to 4 directed FMAs per
 * inner step).  A, B 16-byte aligned (_dev form). */
int vcpcu_igemm_fma_dev(int m, int n, int k, const double* A, int lda,
                        const double* B, int ldb, double* C, int ldc, void* stream);
int vcpcu_igemm_fma(int m, int n, int k, const double* A, const double* B, double* C);

/* ---- autotuner ------------------------------------------------------------- */

/* VCPCU_FORM_AUTO runs, per product, the form with the smaller predicted
 * time: plain 8mnk/fp64_rate + t_launch against Ozaki (L + 8) 2 Mp Np Kp /
 * tc_rate + 16 (mk + kn) / prep_bw + 12 t_launch (L moduli, tile-padded
 * sizes).  vcpcu_autotune measures the constants on the current device
 * (one plain and two Ozaki products on synthetic data), keeps them for the
 * process, stores them in the file named by the environment variable
 * VCPCU_AUTOTUNE_CACHE (read back at the first AUTO decision of a later
 * process), and writes {fp64_rate, tc_rate, prep_bw, t_launch} to
 * constants[4] if non-NULL.  No counterpart in the reference.
 * vcpcu_autotune_choice returns the form AUTO would use for m x n x k, as
 * a single product (batched = 0) or as one problem of a batch (batched != 0:
 * the batch's grouped launches carry no per-product launch cost). */
int vcpcu_autotune(void* stream, double* constants);

/* The AUTO decision for a product C = [A] [B] (A m x k, B k x n, kv layout,
 * host or device pointers): *form = VCPCU_FORM_PLAIN or VCPCU_FORM_OZAKI
 * and *slices the tensor-core slice count, chosen per (inner dimension,
 * exponent spread, radius size) as the first of 6, 7, 8, 9 with
 * VCPCU_SLICES_FAST_RADIUS added, then 8 and 9 without it, whose
 * enclosures a probe finds no wider than the plain form's -- the probe
 * multiplies a block of up to 64 rows of A and up to 64 evenly spaced
 * columns of B in the plain form and at every candidate and compares the
 * widths (the largest sampled ratio below 1 by at least 2^-16 and by a
 * fifth of its distance from the 90th percentile, and at most 1/2 where it
 * exceeds 4 x the median) -- or the plain form when none qualifies;
 * choices are kept for the process (vcpcu_autotune forgets them).  Replaces the reference's
 * fixed split geometry of pddblas_assist::split_shift / max_slices
 * (vcp/pddblas.hpp:54-78), which ignores the width.  Synchronises the
 * stream. */
int vcpcu_autotune_pick(int m, int n, int k, const double* A, int lda, const double* B,
                        int ldb, int* form, int* slices, void* stream);
int vcpcu_autotune_choice(int m, int n, int k, int batched);

/* ---- batches of uneven interval GEMMs -------------------------------------- */

/* One problem of a batch: C (m x n) = [A] (m x k) * [B] (k x n), kv-layout
 * interval matrices, device pointers, column-major with leading dimensions. */
typedef struct {
  int m, n, k;
  int lda, ldb, ldc;
  const double* A;
  const double* B;
  double* C;
} vcpcu_problem;

/* Runs `count` independent interval products (the many small, uneven
 * products that Newton / verification steps and the Legendre basis
 * generator of the reference emit; no single reference entry point: each
 * would be a pidblas::mulmm call).  Form PLAIN: one persistent grouped
 * launch over all problems' 64 x 64 tiles (work counter, no waits),
 * bit-identical per problem to vcpcu_igemm_dev PLAIN.  Form OZAKI: grouped
 * products -- the problems bucketed by padded inner dimension, nine launches
 * per bucket over all its problems -- bit-identical per problem to
 * vcpcu_igemm_dev OZAKI.  OZAKI_SLICES: product by product on forked
 * streams.  AUTO: each problem in the form the cost model picks for a batch
 * problem (vcpcu_autotune_choice with batched = 1), both parts concurrent.
 * The tensor-core forms need 16-byte aligned A and B.  The table is read
 * from host memory during the call; the call plans the grouped products and
 * uploads their tables (it synchronises the stream once, so it cannot run
 * inside a stream capture: use the batch graphs below). */
int vcpcu_igemm_batched_dev(int count, const vcpcu_problem* problems, int form,
                            int slices, void* stream);

/* The same batch captured once into an instantiated CUDA graph (the problem
 * table is copied; its device pointers must stay valid), replayed with one
 * launch per call, with device clock stamps per problem: after a replay,
 * vcpcu_batch_graph_latencies synchronises `stream` and writes, per
 * problem, its start relative to the batch's first start and its latency
 * (first tile start to last tile end for PLAIN, call start to end for the
 * Ozaki forms), in microseconds (either pointer may be NULL). */
typedef struct vcpcu_batch_graph_s* vcpcu_batch_graph;
int vcpcu_batch_graph_create(int count, const vcpcu_problem* problems, int form,
                             int slices, void* stream, vcpcu_batch_graph* out);
int vcpcu_batch_graph_launch(vcpcu_batch_graph g, void* stream);
int vcpcu_batch_graph_latencies(vcpcu_batch_graph g, void* stream,
                                double* start_us, double* latency_us);
int vcpcu_batch_graph_destroy(vcpcu_batch_graph g);

/* ---- double-double GEMM (pddblas::mulmm, vcp/pddblas.hpp:318-376) --------- */

/* C = A * B for kv::dd matrices (pairs {a1, a2} of doubles, column-major;
 * A m x k, B k x n, C m x n) -- replaces pddblas::mulmm and, with A^T as
 * the left factor, pddblas::mulltmm (:379-409).  Each dd entry is scaled
 * per row (A) / column (B) to a w-bit integer, w = 8 * slices (7 <= slices
 * <= 14; 0 = default 14, w = 112 -- the most the 32 moduli carry; lowered
 * for very long k); the integer
 * product is exact (residues modulo up to 32 moduli <= 256 on the bf16
 * tensor cores, Chinese remaindering in 256-bit arithmetic) and is rounded
 * to the dd C = c.a1 + c.a2 (round to nearest, then the exact remainder to
 * nearest).  If Cerr != NULL it receives a rigorous upper bound of
 * |A B - C| per entry (ld lde): the truncation of the operands to w bits,
 * k 2^(E_i + F_j - w) (1 + 2^-40), plus the conversion error; +Inf marks
 * entries whose scaling leaves the normal double range.  Non-finite inputs
 * make every output NaN (VCPCU_ERR_NONFINITE from the host form, or
 * vcpcu_status).  A and B must be 16-byte aligned. */
int vcpcu_ddgemm_dev(int m, int n, int k, const double* A, int lda,
                     const double* B, int ldb, double* C, int ldc, double* Cerr,
                     int lde, int slices, void* stream);
int vcpcu_ddgemm(int m, int n, int k, const double* A, const double* B,
                 double* C, double* Cerr, int slices);

/* ---- interval GEMM without device allocation ------------------------------ */

/* Size of the static device scratch used by vcpcu_igemm_noalloc_dev. */
#define VCPCU_NOALLOC_SCRATCH_BYTES (32u << 20)

/* The Ozaki-form interval product (same kernels and same results as
 * vcpcu_igemm_dev with form VCPCU_FORM_OZAKI and the same `slices`) for
 * callers that must not allocate device memory: a real-time loop that must
 * not reach cudaMalloc (it can synchronise the device), a process whose
 * device memory belongs to another allocator (whose budget an allocation
 * here would overrun), or an FFI caller that promises no allocation after
 * start-up.  No counterpart in the reference (the
 * reference is CPU code and allocates with std::vector).
 *
 * Scratch is one static 32 MiB (VCPCU_NOALLOC_SCRATCH_BYTES) device array
 * that every device loading this library holds until the process exits;
 * problems whose scratch would exceed it (about m = n = k = 400 at the
 * default precision) are rejected with VCPCU_ERR_INVALID_ARG.  No cudaMalloc, cudaFree
 * or allocating library routine is called.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture.  All
 * calls share the array: calls whose GPU work overlaps (different streams,
 * or unordered host threads) race and give wrong results -- order them on
 * one stream.  Device pointers; stream-ordered; returns before the GPU
 * finishes.  Non-finite inputs, or a bounded device wait that gave up,
 * make every output entry NaN. */
int vcpcu_igemm_noalloc_dev(int m, int n, int k, const double* A, int lda,
                            const double* B, int ldb, double* C, int ldc,
                            int slices, void* stream);

/* The verification of imats::eigsymge (vcp/imats.hpp:419-522; Miyajima's
 * enclosure of every eigenvalue of A x = lambda B x, A, B symmetric n x n
 * interval, mid B positive definite) around the approximate eigenvectors X
 * (n x n) and eigenvalues lambda (n) of the midpoint problem, which the
 * reference takes from LAPACK dsygv on the host (:427-434):
 *   stage 1: C = [A] X, BX = [B] X (kv layout, ld n) and mid(BX) (ld n);
 *   the caller forms Y = inv(mid(BX)) (the reference: pdblas::inv);
 *   stage 2: C -= BX diag(lambda); R = Y C; S = Y BX - I; from their norms
 *   and |R| e, |S| e the enclosures lam[2i], lam[2i+1] (before the overlap
 *   merge) and *bound = sup ||S|| (the reference throws
 *   vcp::verification_error when it is >= 1).
 * Every step uses the reference's kv operation; in the plain form R = Y C is
 * the base class's term-by-term kv loop, as in the reference, so all bits
 * match it (for n >= 2); the tensor-core forms enclose the same products.
 * Device pointers; C is overwritten by stage 2; lam, bound in device memory.
 * vcpcu_eig_merge is the reference's final overlap merge (host memory).
 * vcpcu_ieigsymge (host memory) runs both stages, calls inv(n, M, ctx) to
 * turn M = mid(BX) (column-major) into its inverse in place (non-zero
 * return: VCPCU_ERR_INVALID_ARG), merges, and returns VCPCU_ERR_VERIFY
 * when *bound >= 1 (lam then meaningless). */
typedef int (*vcpcu_inverse_fn)(int n, double* M, void* ctx);
int vcpcu_ieigsymge_stage1_dev(int n, const double* A, int lda, const double* B, int ldb,
                               const double* X, int ldx, double* C, double* BX, double* midBX,
                               int form, int slices, void* stream);
int vcpcu_ieigsymge_stage2_dev(int n, const double* lambda, const double* Y, int ldy, double* C,
                               const double* BX, double* lam, double* bound, int form,
                               int slices, void* stream);
int vcpcu_eig_merge(int n, double* lam);
int vcpcu_ieigsymge(int n, const double* A, const double* B, const double* X,
                    const double* lambda, vcpcu_inverse_fn inv, void* ctx, double* lam,
                    double* bound, int form, int slices);

/* ---- portable matrix files (vcp/vcp_portable_fio.hpp) ----------------- */

/* Element types of a .vcpmat file (vcp/vcp_portable_fio.hpp:60-66) and their
 * in-memory layout (column-major, one element after the other). */
#define VCPCU_MAT_INT32       1  /* int32                                      */
#define VCPCU_MAT_DOUBLE      2  /* double                                     */
#define VCPCU_MAT_INTERVAL    3  /* kv::interval<double>: {lower, upper}        */
#define VCPCU_MAT_DD          4  /* kv::dd: {a1, a2}                            */
#define VCPCU_MAT_INTERVAL_DD 5  /* kv::interval<kv::dd>: {lo.a1, lo.a2, up.a1, up.a2} */

/* <name>.vcpmat in the format of vcp::save_portable / load_portable
 * (vcp/vcp_portable_fio.hpp:476-565): same bytes as the reference writes,
 * written through <name>.vcpmat.tmp and a rename; a load checks magic,
 * version, layout, type, sizes, CRC-64 and trailing data and returns
 * VCPCU_ERR_IO where the reference throws vcp::io_error.  rows and cols must
 * match the file (vcpcu_vcpmat_info reads them); 0 x 0 is allowed.  The
 * _dev forms stream the matrix to / from device memory (leading dimension
 * ld, in elements) through pinned chunks on `stream` and return after it. */
int vcpcu_vcpmat_save(const char* name, int type, int rows, int cols, const void* data);
int vcpcu_vcpmat_info(const char* name, int* type, int* rows, int* cols);
int vcpcu_vcpmat_load(const char* name, int type, int rows, int cols, void* data);
int vcpcu_vcpmat_save_dev(const char* name, int type, int rows, int cols, const void* ddata,
                          int ld, void* stream);
int vcpcu_vcpmat_load_dev(const char* name, int type, int rows, int cols, void* ddata, int ld,
                          void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VCPCUDA_H */
