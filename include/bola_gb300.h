/*
 * bola_gb300.h — C ABI of the GB300 (sm_103a) implementation of BOLA's dense
 * BLAS-3/LAPACK path.
 *
 * Conventions (those of BOLA, alexlovric/bola v0.1.2):
 *   - column-major FP64 matrices, leading dimensions in elements;
 *   - ipiv is 1-based int32 (row i was swapped with row ipiv[i]); idamax is 0-based;
 *   - every matrix/vector pointer is a DEVICE pointer; scalars are host values;
 *   - `stream` is a cudaStream_t (NULL = the legacy default stream); the call
 *     enqueues its work on it and returns without waiting for the GPU;
 *   - return value: 0 success; -i argument i is illegal (LAPACK numbering, the
 *     arguments BOLA itself checks); values <= -1000 are BOLA_ERR_* below, with
 *     a message from bola_last_error().  Factorisation failures that the GPU
 *     discovers (zero pivot, matrix not positive definite) are written to the
 *     device int32 *info as a 1-based global column, 0 when the factorisation
 *     succeeded; the factorisation stops at that column as BOLA does.
 *   - characters are accepted in either case with their BLAS meaning.
 *
 * Rounding: each routine performs, element for element, the same sequence of
 * IEEE operations as BOLA's CPU code (same blocking, same fused/unfused
 * multiply-adds), so results are bit-identical to BOLA's for the SIMD width
 * selected by bola_set_simd_lanes (2 = BOLA built for aarch64/NEON, the
 * default; 4 = BOLA built for x86_64/AVX2).
 */
#ifndef BOLA_GB300_H
#define BOLA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void *bola_stream_t; /* cudaStream_t */

#define BOLA_OK 0
#define BOLA_ERR_CUDA (-1000)        /* a CUDA runtime call failed */
#define BOLA_ERR_NO_DEVICE (-1001)   /* no usable sm_103 device */
#define BOLA_ERR_UNSUPPORTED (-1002) /* argument combination outside this library */
/* Device-side *info of bola_dgetrf / bola_dgetrf2: a panel's bounded wait for
 * another CTA of its cluster expired (the factor is unusable; the context
 * stays usable).  Positive values keep their meaning (first zero pivot). */
#define BOLA_INFO_WAIT_EXPIRED (-2000)

/* Library identification and diagnostics. */
const char *bola_version(void);
const char *bola_last_error(void); /* message of this thread's last failing call */

/* Which of BOLA's two SIMD builds to reproduce bit-for-bit: 2 (aarch64 NEON,
 * default) or 4 (x86_64 AVX2).  Returns the previous value, or -1 if invalid. */
int bola_set_simd_lanes(int lanes);
int bola_get_simd_lanes(void);

/* Device-time profiler: the GPU counterpart of BOLA's `profiling` feature
 * (src/profiling.rs:25-140).  While enabled, every kernel launch is bracketed
 * by CUDA events on its stream and tagged with a routine name plus its
 * algorithmic flop/byte counts.  bola_profile_count() waits for the recorded
 * events and returns the number of routine names seen; bola_profile_read()
 * returns one name's totals (scopes, kernel launches, device ms, flops, bytes). */
int bola_profile_enable(int on); /* returns the previous setting */
int bola_profile_reset(void);
int bola_profile_count(void);
int bola_profile_read(int index, char *name, int name_len, int64_t *calls, int64_t *launches, double *ms,
                      double *flops, double *bytes);

/* Measures this device's FP64 fused multiply-add throughput (GFLOP/s) with a
 * ~20 ms register-resident DFMA loop over every SM, so that roofline
 * fractions of the FP64 kernels are stated against a peak measured on the
 * same device and clocks.  Synchronises the device. */
int bola_measure_fp64_peak(double *gflops);

/* The same FP64 throughput measurement through the tensor cores' FP64 MMA
 * (mma.sync m8n8k4 f64, eight independent tiles per warp, every SM), so the
 * choice of DFMA for the FP64 kernels rests on a measurement on this device.
 * Synchronises the device.  No BOLA counterpart. */
int bola_measure_dmma_peak(double *gflops);

/* Measures one exchange round of a cluster panel (no BOLA counterpart): csize
 * (1..16) CTAs each copy `bytes` (16..8192, a multiple of 16) of shared memory
 * into every CTA of the cluster with bulk copies that complete on the
 * receiver's mbarrier, then wait for their own arrivals (bounded) and meet a
 * CTA barrier.  *us_per_round gets the time per round (microseconds), the
 * floor of the mixed LU panels' serial chain per pivot group.  Synchronises
 * the device. */
int bola_measure_cluster_exchange(int csize, int bytes, double *us_per_round);

/* Self-test of the library's bounded waits (no BOLA counterpart): one kernel
 * waits on an mbarrier that nothing completes and on a device flag that
 * nothing sets (flag_err[1], which must be 0), each for at most `polls`
 * polls, and ORs 1 (mbarrier) and 2 (flag) into flag_err[0] when it gives
 * up — the path every panel, tensor-core pipeline and dataflow solve takes
 * when a wait expires.  The kernel returns normally; the context stays
 * usable.  Asynchronous on the stream. */
int bola_selftest_bounded_waits(int32_t *flag_err, uint32_t polls, bola_stream_t stream);

/* ---- Level 1 ---------------------------------------------------------- */

/* Replaces idamax(n, x) -> usize, src/idamax.rs:23 (x86_64) / :141 (aarch64).
 * Writes the 0-based index of the element of largest |x| (BOLA's lane-merge
 * order on ties; NaN never selected) to the device int64 *result. */
int bola_idamax(int64_t n, const double *x, int64_t *result, bola_stream_t stream);

/* Replaces scal(n, alpha, x, incx), src/scal.rs:45. */
int bola_dscal(int64_t n, double alpha, double *x, int64_t incx, bola_stream_t stream);

/* Replaces ger(m, n, alpha, x, y, ldy, a, lda), src/ger.rs:28:  A += alpha x y^T,
 * x contiguous, y with stride ldy. */
int bola_dger(int64_t m, int64_t n, double alpha, const double *x, const double *y, int64_t ldy,
              double *a, int64_t lda, bola_stream_t stream);

/* Replaces dot_product(n, x, incx, y, incy) -> f64, src/utilities.rs:22 / :62.
 * Writes the result to the device double *result. */
int bola_ddot(int64_t n, const double *x, int64_t incx, const double *y, int64_t incy,
              double *result, bola_stream_t stream);

/* Replaces daxpy(n, alpha, x, incx, y, incy), src/utilities.rs:107 / :140. */
int bola_daxpy(int64_t n, double alpha, const double *x, int64_t incx, double *y, int64_t incy,
               bola_stream_t stream);

/* Replaces laswp(n, a, lda, k1, k2, ipiv, incx), src/laswp.rs:22.  ipiv is a
 * device int32 array indexed like BOLA's slice (k1, k2 1-based). */
int bola_dlaswp(int64_t n, double *a, int64_t lda, int32_t k1, int32_t k2, const int32_t *ipiv,
                int32_t incx, bola_stream_t stream);

/* ---- BLAS 3 ----------------------------------------------------------- */

/* Replaces gemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc),
 * src/gemm.rs:88:  C = alpha op(A) op(B) + beta C. */
int bola_dgemm(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
               const double *a, int64_t lda, const double *b, int64_t ldb, double beta, double *c,
               int64_t ldc, bola_stream_t stream);

/* Replaces trsm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb),
 * src/trsm.rs:33:  op(A) X = alpha B (side 'L') or X op(A) = alpha B ('R'), X over B. */
int bola_dtrsm(char side, char uplo, char transa, char diag, int64_t m, int64_t n, double alpha,
               const double *a, int64_t lda, double *b, int64_t ldb, bola_stream_t stream);

/* Replaces syrk(uplo, trans, n, k, alpha, a, lda, beta, c, ldc), src/syrk.rs:17:
 * C = alpha A A^T + beta C ('N') or alpha A^T A + beta C ('T'), one triangle.
 * (uplo,trans) = (L,N) and (U,T) are bit-identical to BOLA; (U,N) and (L,T)
 * compute the BLAS definition (BOLA addresses A wrongly there once n or k
 * exceeds 32, src/syrk.rs:80,139). */
int bola_dsyrk(char uplo, char trans, int64_t n, int64_t k, double alpha, const double *a,
               int64_t lda, double beta, double *c, int64_t ldc, bola_stream_t stream);

/* DGEMM that allocates no device memory.  No counterpart in BOLA: it exists
 * for callers of this library that cannot allocate — code running where
 * cudaMalloc and memory-pool calls are not allowed or not wanted (inside a
 * real-time loop where an allocation could stall, under an application that
 * owns all device memory through its own allocator, or with a memory budget
 * that must not move).  Same arguments and bit-identical results as
 * bola_dgemm.  Where bola_dgemm would borrow temporary memory for its split-K
 * partial sums (outputs too small to fill the GPU), this call uses a fixed
 * 64 MiB array compiled into the library instead; every GPU that loads the
 * library holds that array until the process exits.
 *   - Shapes whose split-K partial sums need more than 64 MiB (K/64 chunks x
 *     m x n doubles, rounded as bola_dgemm rounds them) are rejected with
 *     BOLA_ERR_UNSUPPORTED and a message in bola_last_error().
 *   - The first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.  The address is cached with the id of the
 *     device's context: after a device reset the first call in the new
 *     context looks it up again, and that call too belongs before any
 *     capture.
 *   - All calls on a device share the one array: calls whose kernels can
 *     overlap on the GPU (different streams, no ordering) race on it.  Calls
 *     on one stream are safe; each call writes every scratch value it later
 *     reads, so nothing carries over from the previous call. */
#define BOLA_NOALLOC_SCRATCH_BYTES (64ull << 20)
int bola_dgemm_noalloc(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
                       const double *a, int64_t lda, const double *b, int64_t ldb, double beta,
                       double *c, int64_t ldc, bola_stream_t stream);

/* Building block of the mixed-precision solver (no BOLA counterpart):
 * W (m x n FP32, column-major) -= A * B^T on the tcgen05 tensor cores, A
 * (m x 64) and B (n x 64) stored K-major (64 contiguous values per row).
 * kind 0: bf16 operands; 1: tf32 operands (fp32 storage); 2: 3xTF32, with
 * a_lo/b_lo the tf32 remainders (A ~ a + a_lo), for ~2^-22 relative accuracy.
 * *err (device int32) becomes non-zero if a bounded on-chip wait expired. */
int bola_sgemm_tc_update(int kind, int64_t m, int64_t n, const void *a, const void *b, const void *a_lo,
                         const void *b_lo, float *w, int64_t ldw, int32_t *err, bola_stream_t stream);

/* The low-precision LU of bola_dgesv_mixed alone (no BOLA counterpart;
 * exposed for testing and profiling): W (n x n FP32, column-major, ld ldw,
 * n <= 8192) is replaced by P W = L U (unit-lower L below the diagonal, U on
 * and above), blocked right-looking with 64-column panels whose pivots are
 * chosen by tournament (8-column groups) and tcgen05 trailing updates of the
 * given kind (0 bf16, 1 tf32, 2 3xTF32).  ipiv (device, n entries) gets
 * LAPACK-style 1-based interchanges, *info (device) the first exact-zero
 * pivot (1-based) or 0.  Synchronous. */
int bola_sgetrf_mixed(int kind, int64_t n, float *w, int64_t ldw, int32_t *ipiv, int32_t *info,
                      bola_stream_t stream);

/* The low-precision Cholesky of bola_dposv_mixed alone (no BOLA counterpart;
 * exposed for testing and profiling): the lower triangle of W (n x n FP32 SPD,
 * ld ldw, n <= 8192) is replaced by L, W = L L^T, with tcgen05 trailing
 * updates of the given kind (0 bf16, 1 tf32, 2 3xTF32).  *info (device) =
 * the first column whose pivot is not positive (1-based), or 0.  Synchronous. */
int bola_spotrf_mixed(int kind, int64_t n, float *w, int64_t ldw, int32_t *info, bola_stream_t stream);

/* FP64-accurate matrix product on the bf16 tensor cores (no BOLA
 * counterpart; the residuals and GMRES products of bola_dgesv_mixed, exposed
 * for testing and profiling): out = b - A x, or out = A x when b is NULL,
 * with A n x n and x, b, out n x nrhs (FP64, column-major).  A is split
 * exactly into 7 planes of 8-bit digits under a power-of-two scale per row,
 * x into 8 planes under a scale per column; every plane pair of weight
 * 2^-56 or more is accumulated exactly (integer partial sums in FP32 on
 * tcgen05, combined in 64-bit fixed point).  Error per element at most about
 * 2^-54 n max_j|a_ij| max|x_c| + 2^-52 |(A x)_ic| (the roundings of the
 * digits and of the final FP64 sum); a row of A or a column of x holding an
 * Inf or NaN gives NaN.  Allocates its digit planes per call; synchronous. */
int bola_dgemv_oz(int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *x, int64_t ldx,
                  const double *b, int64_t ldb, double *out, int64_t ldo, bola_stream_t stream);

/* FP64-accurate update on the bf16 tensor cores (no BOLA counterpart; the
 * trailing update of factor_kind 3 of bola_dgesv_mixed, exposed for
 * testing):  W (m x n, FP64, column-major, ld ldw) -= A B^T with A (m x 64)
 * and B (n x 64) FP64, stored K-major (64 contiguous K values per row).
 * Each row of A and B is split exactly into six 8-bit integer slices under a
 * power-of-two scale; slice products accumulate exactly in FP32 on the
 * tensor cores and are combined in FP64.  Error per element about
 * 2^-46 * 64 * max|A row| * max|B row|.  *err (device) is set non-zero if a
 * bounded wait inside the kernel expired. */
int bola_dgemm_oz_update(int64_t m, int64_t n, const double *a, const double *b, double *w, int64_t ldw,
                         int32_t *err, bola_stream_t stream);

/* ---- LAPACK ----------------------------------------------------------- */

/* Replaces getrf(m, n, a, lda, ipiv) -> Result, src/getrf.rs:37.  Returns -4 for
 * lda < max(1, m) (BOLA: "Argument 4 to getrf had an illegal value").  *info
 * (device) = 0, or the 1-based column whose pivot is exactly zero (BOLA:
 * "Matrix is singular..."), in which case A and ipiv stay as BOLA leaves them. */
int bola_dgetrf(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv, int32_t *info,
                bola_stream_t stream);

/* Replaces getrf2(m, n, a, lda, ipiv) -> Result, src/getrf2.rs:39 (recursive LU). */
int bola_dgetrf2(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv, int32_t *info,
                 bola_stream_t stream);

/* Replaces potrf(uplo, n, a, lda) -> Result, src/potrf.rs:101.  Returns -1 for
 * uplo other than 'U'/'L' (BOLA requires upper case here), -4 for
 * lda < max(1, n).  *info (device) = 0 or the 1-based column where A is found
 * not positive definite. */
int bola_dpotrf(char uplo, int64_t n, double *a, int64_t lda, int32_t *info, bola_stream_t stream);

/* Replaces potrf2(uplo, n, a, lda) -> Result, src/potrf2.rs:25 (recursive Cholesky). */
int bola_dpotrf2(char uplo, int64_t n, double *a, int64_t lda, int32_t *info, bola_stream_t stream);

/* Solve with the LU factors of bola_dgetrf: laswp on B, then unit-lower and
 * upper triangular solves — the composite BOLA users write by hand (BOLA has
 * no getrs; src/laswp.rs:22 + src/trsm.rs:95,135).  B (n x nrhs) is overwritten. */
int bola_dgetrs(int64_t n, int64_t nrhs, const double *lu, int64_t lda, const int32_t *ipiv,
                double *b, int64_t ldb, bola_stream_t stream);

/* Solve with the Cholesky factor of bola_dpotrf (uplo 'L': L then L^T solves,
 * src/trsm.rs:95,174; 'U': U^T then U, src/trsm.rs:213,135). */
int bola_dpotrs(char uplo, int64_t n, int64_t nrhs, const double *fac, int64_t lda, double *b,
                int64_t ldb, bola_stream_t stream);

/* ---- Mixed-precision solve (no BOLA counterpart) ------------------------
 * Solves A X = B (A n x n FP64, B and X n x nrhs FP64, device pointers) to a
 * normwise backward error max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf
 * + ||b_j||_inf) <= tolerance: A is factored in low precision (FP32 storage,
 * tcgen05 tensor-core trailing updates, per-64-column-block power-of-two
 * scaling), then the solution is refined with FP64 residuals and updates.
 * Plain refinement runs while each sweep cuts the backward error by 20x or
 * more; otherwise flexible GMRES on the correction equation, preconditioned
 * by the low-precision LU, takes over (GMRES-IR); if that stalls too, the
 * plain FP64 path (bola_dgetrf + bola_dgetrs) solves the system, when
 * fallback_fp64 is set.  The FP64 path is taken at once when the spread
 * max|u_ii| / min|u_ii| of the low-precision U exceeds a per-kind limit
 * (bf16 175, tf32 1100, 3xTF32 4.5e4), beyond which refinement was measured
 * not to converge.  Synchronous: it
 * returns after the result and *info are final.  n <= 8192, nrhs <= 32. */
typedef struct {
  int factor_kind;       /* 0: bf16 tensor-core updates; 1: tf32; 2: 3xTF32 (FP32-accurate);
                            3: FP64 storage, exact-split bf16 tensor-core updates (FP64-accurate) */
  int max_iterations;    /* refinement sweeps before declaring a stall (default 30) */
  double tolerance;      /* target backward error (default 1e-14) */
  int fallback_fp64;     /* 1: finish with the plain FP64 path when refinement stalls */
  int gmres;             /* 1: switch to GMRES-IR when plain refinement is slow (< 20x per sweep) or stalls */
  int escalate;          /* 1: when a factor of kind 0-2 cannot reach the tolerance, solve again with
                            kind 3 before the FP64 fallback */
} bola_mixed_opts;

typedef struct {
  int iterations;        /* refinement sweeps performed */
  int gmres_iterations;  /* inner GMRES steps (GMRES-IR), 0 when not used */
  int path;              /* 0 mixed IR, 1 mixed GMRES-IR, 2 plain FP64 fallback,
                            3 escalated to factor kind 3 and refined there */
  int factor_info;       /* first zero pivot of the low-precision LU (1-based), 0 if none */
  double backward_error; /* of the returned X */
  double condition_estimate; /* max|u_ii| / min|u_ii| of the low-precision factor */
  int factorization;     /* the factor the answer was refined with: 0 LU, 1 Cholesky */
  int reserved;
} bola_mixed_info;

int bola_dgesv_mixed(int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *b, int64_t ldb,
                     double *x, int64_t ldx, const bola_mixed_opts *opts, bola_mixed_info *info,
                     bola_stream_t stream);

/* Mixed-precision solve of a symmetric positive definite system (no BOLA
 * counterpart; the FP64 answer it must reach is BOLA's potrf('L') + potrs
 * solve, src/potrf.rs:101-181).  A is n x n SPD, stored in full (the
 * factorisation reads its lower triangle, the FP64 residuals all of it).
 * W = fl(D A D) with D a power of two per row (unit-order diagonal) is
 * factored W = L L^T on the tensor cores (64-column panels: the diagonal
 * block in one CTA, L21 as a parallel triangular solve, no pivoting; the
 * trailing update W22 -= L21 L21^T only on tiles reaching the diagonal),
 * then refined in FP64 exactly as bola_dgesv_mixed refines (IR, GMRES-IR,
 * escalation to the FP64-accurate factor kind 3, here a Cholesky too).  A
 * pivot that is not positive means A is not SPD at the factor's precision:
 * the call then solves with the mixed LU (info->factorization = 0).  Same
 * options, limits and return codes as bola_dgesv_mixed. */
int bola_dposv_mixed(int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *b, int64_t ldb,
                     double *x, int64_t ldx, const bola_mixed_opts *opts, bola_mixed_info *info,
                     bola_stream_t stream);

/* The same solve with caller-owned device workspace, so that several solves
 * can run at once on different streams and host threads (bola_dgesv_mixed
 * shares one workspace per device and serialises).  A context grows to the
 * largest (n, nrhs) it has served; bola_mixed_ctx_bytes reports its size. */
typedef struct bola_mixed_ctx_st *bola_mixed_ctx;
int bola_mixed_ctx_create(bola_mixed_ctx *ctx);
int bola_mixed_ctx_destroy(bola_mixed_ctx ctx);
int64_t bola_mixed_ctx_bytes(bola_mixed_ctx ctx);
int bola_dgesv_mixed_ctx(bola_mixed_ctx ctx, int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *b,
                         int64_t ldb, double *x, int64_t ldx, const bola_mixed_opts *opts, bola_mixed_info *info,
                         bola_stream_t stream);
int bola_dposv_mixed_ctx(bola_mixed_ctx ctx, int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *b,
                         int64_t ldb, double *x, int64_t ldx, const bola_mixed_opts *opts, bola_mixed_info *info,
                         bola_stream_t stream);

/* ---- Batched solves of many small systems (no BOLA counterpart) --------
 * Each system: A X = B with A n x n (1 <= n <= 256), kind 0 = general (LU
 * with partial pivoting), kind 1 = symmetric positive definite (Cholesky,
 * lower triangle used); A is overwritten by its factors and B by X.  All
 * systems of a batch are solved in ONE persistent kernel launch: a plan
 * buckets the systems by n, gives each bucket a group size (threads per
 * system, from an autotuned table or the built-in defaults) and orders the
 * work largest first.  Results do not depend on which other systems are in
 * the batch.  info[i] (device) = 0, or the 1-based column of a zero pivot
 * (kind 0) or of the first non-positive pivot (kind 1). */
typedef struct {
  int32_t n, nrhs, kind, lda, ldb, reserved;
  double *a; /* device, n x n column-major */
  double *b; /* device, n x nrhs column-major */
} bola_system;

typedef struct bola_batch_plan_st *bola_batch_plan;

/* n, kind: host arrays of `count`.  group_size: host array of 8 group sizes
 * (32/64/128/256) for the buckets n <= 16, 32, 48, 64, 96, 128, 192, 256;
 * NULL = built-in defaults.  Returns -2 for an n outside 1..256. */
int bola_batch_plan_create(int32_t count, const int32_t *n, const int32_t *kind, const int32_t *group_size,
                           bola_batch_plan *plan);

/* The tuning table of the batched solver, per size bucket (n <= 16, 32, 48,
 * 64, 96, 128, 192, 256): group_size = threads per system (32/64/128/256),
 * panel_width = columns per factorisation panel (8/12/16); and tile_rows =
 * rows of the per-thread register tile of the trailing updates (4 or 2,
 * with 4 columns), one value per plan because it sets the kernel's register
 * count.  Zero entries take the built-in defaults (group sizes 32..256 by
 * bucket, panel width 8, tile 4).  None of the three changes any system's
 * operation order: a tuned plan gives bit-identical results. */
typedef struct {
  int32_t group_size[8];
  int32_t panel_width[8];
  int32_t tile_rows;
  int32_t reserved;
} bola_batch_tuning;
/* bola_batch_plan_create with a full tuning table (NULL = defaults); -4 for a
 * tile_rows other than 0, 2 or 4. */
int bola_batch_plan_create_tuned(int32_t count, const int32_t *n, const int32_t *kind,
                                 const bola_batch_tuning *tuning, bola_batch_plan *plan);
/* Writes / reads a tuning table as JSON ({"group_size": [...], "panel_width":
 * [...], "tile_rows": r, "device": name, "sms": count}).  The loader checks
 * every value and returns -2 for a file it cannot read or parse, -3 for a
 * table whose values are out of range; *sms_recorded (may be NULL) gets the
 * SM count of the device the table was measured on. */
int bola_batch_tuning_save(const char *path, const bola_batch_tuning *tuning);
int bola_batch_tuning_load(const char *path, bola_batch_tuning *tuning, int32_t *sms_recorded);
/* systems: device array of `count` descriptors; info: device int32[count]. */
int bola_batch_solve(bola_batch_plan plan, const bola_system *systems, int32_t *info, bola_stream_t stream);
/* Same solve through a CUDA graph captured on first use for these pointers
 * and replayed afterwards (one graph launch per batch). */
int bola_batch_solve_graph(bola_batch_plan plan, const bola_system *systems, int32_t *info,
                           bola_stream_t stream);
int bola_batch_plan_info(bola_batch_plan plan, int32_t *nitems, int32_t *grid, double *flops);
int bola_batch_plan_destroy(bola_batch_plan plan);

/* ---- Solve server (no BOLA counterpart) --------------------------------
 * Accepts solve requests A X = B (host buffers, column-major, ld = n;
 * 1 <= n <= 8192, 1 <= nrhs <= 32; kind 0 general, 1 SPD) from any host
 * thread and serves them on the current device.  Requests are admitted in
 * arrival order while the device bytes held by admitted requests stay within
 * hbm_budget_bytes.  Requests with n > small_n run on `slots` workers, each
 * with its own stream and mixed-solver context (several run at once); in
 * mode 0 they take bola_dgesv_mixed_ctx (tensor-core LU, FP64 refinement,
 * FP64 fallback), or bola_dposv_mixed_ctx for SPD requests (kind 1: the
 * tensor-core Cholesky, the same refinement), in mode 1 the plain
 * FP64 path (bola_dgetrf/bola_dgetrs, or bola_dpotrf/bola_dpotrs for SPD).
 * Requests with n <= small_n (at most 256) are gathered continuously: every
 * admitted small request waiting when the previous batch ends goes into the
 * next persistent batched launch (bola_batch_solve, FP64).  Every result's
 * normwise backward error is measured in FP64 on the device against the
 * request's original A and B.  A result does not depend on the other
 * requests in flight.  The caller keeps a and b alive until the request's
 * bola_server_wait returns. */
typedef struct {
  int32_t slots;        /* concurrent large-request workers (>= 1) */
  int32_t small_n;      /* largest n sent to the batcher (0..256) */
  int32_t max_batch;    /* most small requests in one batched launch */
  int32_t mode;         /* 0 mixed precision, 1 plain FP64 per request */
  int32_t factor_kind;  /* mode 0: factor kind as in bola_mixed_opts */
  int32_t group_size[8];/* batched group sizes per bucket; all 0 = defaults */
  int32_t reserved;
  int64_t hbm_budget_bytes; /* admission budget for requests' device buffers */
  int32_t panel_width[8];   /* batched panel widths per bucket (bola_batch_tuning); all 0 = default 8 */
  int32_t tile_rows;        /* batched register tile rows (2 or 4); 0 = 4 */
  int32_t reserved2;
} bola_server_opts;

typedef struct {
  int32_t status;        /* 0 queued, 1 running, 2 done; < 0 error code */
  int32_t path;          /* 0 mixed IR, 1 GMRES-IR, 2 FP64, 3 batched FP64,
                            4 escalated to the FP64-accurate factor and refined there */
  int32_t iterations;    /* refinement sweeps (mixed paths) */
  int32_t info;          /* factorisation info (0 = success) */
  double backward_error; /* max over right-hand sides */
  double t_submit, t_admit, t_done; /* seconds since the server was created */
  int32_t factorization; /* 0 LU, 1 Cholesky (the factor the answer came from) */
  int32_t reserved;
} bola_request_info;

typedef struct bola_server_st *bola_server;
int bola_server_create(const bola_server_opts *opts, bola_server *server);
/* Returns -2 for n outside 1..8192, -3 for nrhs outside 1..32, -4 for a kind
 * other than 0/1, -5 when the request alone needs more device bytes than
 * the budget.  *id identifies the request for bola_server_wait. */
int bola_server_submit(bola_server server, int64_t n, int64_t nrhs, int32_t kind, const double *a,
                       const double *b, int64_t *id);
/* Blocks until request `id` is done, copies X (n x nrhs) into x (host, may
 * be NULL) and its record into *info; the id is then released.  Returns the
 * request's error status (0 on success), -2 for an unknown id. */
int bola_server_wait(bola_server server, int64_t id, double *x, bola_request_info *info);
int bola_server_stats(bola_server server, int64_t *bytes_in_use, int32_t *pending, int32_t *running);
/* Serves every request already submitted, then stops the workers. */
int bola_server_destroy(bola_server server);

#ifdef __cplusplus
}
#endif
#endif /* BOLA_GB300_H */
