/*
 * bola_oracle.h — CPU restatement of BOLA's dense BLAS-3/LAPACK routines.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against and the timed CPU baseline; the product library never links it.
 *
 * Every routine restates the algorithm of the Rust crate alexlovric/bola
 * (v0.1.2) with the same blocking constants, loop orders, FMA sites and
 * argument conventions (column-major, 1-based ipiv, 0-based idamax).  Rust
 * never contracts a*b+c, so this file is compiled with -ffp-contract=off and
 * uses fma() exactly where BOLA uses a vector FMA intrinsic.
 *
 * BOLA's SIMD bodies differ between its AVX2 (x86_64) and NEON (aarch64)
 * builds only in the vector width, which decides which elements of a daxpy /
 * ger / dot go through the fused vector body and which through the unfused
 * scalar tail, and how idamax merges lanes.  oracle_set_lanes(4) selects the
 * AVX2 semantics, oracle_set_lanes(2) (the default) the NEON semantics.
 */
#ifndef BOLA_ORACLE_H
#define BOLA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Vector width whose rounding is reproduced: 2 (NEON, default) or 4 (AVX2). */
void oracle_set_lanes(int lanes);
int oracle_get_lanes(void);
/* OpenMP threads used where BOLA uses Rayon (0 = all available). */
void oracle_set_threads(int threads);
int oracle_get_threads(void);

/* Level 1 (src/idamax.rs, src/scal.rs, src/ger.rs, src/utilities.rs). */
int64_t oracle_idamax(int64_t n, const double *x);
int64_t oracle_scal_kernel(int64_t m, double inv_diag, double *col);
void oracle_scal(int64_t n, double alpha, double *x, int64_t incx);
void oracle_ger(int64_t m, int64_t n, double alpha, const double *x, const double *y, int64_t ldy,
                double *a, int64_t lda);
double oracle_dot_product(int64_t n, const double *x, int64_t incx, const double *y, int64_t incy);
void oracle_daxpy(int64_t n, double alpha, const double *x, int64_t incx, double *y, int64_t incy);

/* BLAS-3 (src/gemm.rs, src/trsm.rs, src/syrk.rs). */
void oracle_gemm(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
                 const double *a, int64_t lda, const double *b, int64_t ldb, double beta,
                 double *c, int64_t ldc);
void oracle_trsm(char side, char uplo, char transa, char diag, int64_t m, int64_t n, double alpha,
                 const double *a, int64_t lda, double *b, int64_t ldb);
void oracle_syrk(char uplo, char trans, int64_t n, int64_t k, double alpha, const double *a,
                 int64_t lda, double beta, double *c, int64_t ldc);

/* Row interchanges (src/laswp.rs). */
void oracle_laswp(int64_t n, double *a, int64_t lda, int32_t k1, int32_t k2, const int32_t *ipiv,
                  int32_t incx);

/*
 * LAPACK drivers (src/getrf.rs, src/getrf2.rs, src/potrf.rs, src/potrf2.rs).
 * Return 0 on success.  BOLA returns Err(String); the codes are:
 *   -4            lda illegal            (src/getrf.rs:41-43, src/getrf2.rs:43-45, src/potrf.rs:108-110)
 *   -1            uplo illegal           (src/potrf.rs:105-107)
 *   j > 0         getrf: pivot in column j (1-based) is exactly zero (src/getrf2.rs:166-168)
 *   j > 0         potrf: not positive definite, failing column j (1-based, src/potrf2.rs:31,41-48)
 * On failure the factorisation stops where BOLA stops, leaving A and ipiv
 * partly updated exactly as BOLA leaves them.
 */
int oracle_getrf(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv);
int oracle_getrf2(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv);
int oracle_potrf(char uplo, int64_t n, double *a, int64_t lda);
int oracle_potrf2(char uplo, int64_t n, double *a, int64_t lda);

/*
 * Diagnostic: when non-NULL, every unblocked panel step of getrf writes the
 * relative gap between the largest and second-largest |candidate| of its
 * pivot column to margins[global column].  Used to show that a pivot that
 * differs between two summation orders was a rounding-level near-tie.
 */
void oracle_set_pivot_margins(double *margins, int64_t len);

#ifdef __cplusplus
}
#endif
#endif
