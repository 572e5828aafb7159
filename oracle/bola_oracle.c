/*
 * bola_oracle.c — CPU restatement of BOLA (alexlovric/bola v0.1.2).
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the GPU library and the
 * timed CPU baseline ("BOLA restated in C": Rust is not available to build
 * BOLA itself).  Nothing in the product library links or calls this file.
 *
 * Build with -ffp-contract=off (Rust never fuses a*b+c); fma() marks exactly
 * the sites where BOLA uses _mm256_fmadd_pd / vfmaq_f64.  OpenMP stands in for
 * Rayon at the same loops; every parallel loop writes disjoint elements in the
 * same per-element order as BOLA, so results do not depend on thread count.
 * Each function cites the BOLA source lines it restates (paths relative to
 * the BOLA crate root).
 */
#include "bola_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* The one fused multiply-add BOLA's vector bodies perform (correctly rounded,
 * so the result does not depend on whether the compiler vectorises it). */
#define ORACLE_FMA(a, b, c) fma((a), (b), (c))

static int g_lanes = 2;   /* 2 = NEON semantics, 4 = AVX2 semantics */
static int g_threads = 0; /* 0 = OpenMP default */
static double *g_margins = NULL;
static int64_t g_margins_len = 0;

void oracle_set_lanes(int lanes) { g_lanes = (lanes == 4) ? 4 : 2; }
int oracle_get_lanes(void) { return g_lanes; }
void oracle_set_threads(int threads) { g_threads = threads < 0 ? 0 : threads; }
int oracle_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}
void oracle_set_pivot_margins(double *margins, int64_t len) {
  g_margins = margins;
  g_margins_len = margins ? len : 0;
}

static inline int64_t imin(int64_t a, int64_t b) { return a < b ? a : b; }
static inline int64_t imax(int64_t a, int64_t b) { return a > b ? a : b; }
static inline int is_ch(char c, char upper) { return c == upper || c == (char)(upper + ('a' - 'A')); }

/* ------------------------------------------------------------------------ */
/* Level 1                                                                    */
/* ------------------------------------------------------------------------ */

/* src/idamax.rs:23-133 (AVX2, lanes=4) and :141-240 (NEON, lanes=2).
 * Four accumulators of `lanes` lanes each walk chunks of 4*lanes elements with
 * a strict ordered '>' (NaN never wins); accumulators 1..3 merge into 0 lane
 * by lane, lanes merge left to right, then the scalar tail. */
int64_t oracle_idamax(int64_t n, const double *x) {
  const int L = g_lanes;
  const int64_t small = (L == 4) ? 16 : 8;
  if (n < small) {
    double max_val = -1.0;
    int64_t max_idx = 0;
    for (int64_t i = 0; i < n; i++) {
      double v = fabs(x[i]);
      if (v > max_val) {
        max_val = v;
        max_idx = i;
      }
    }
    return max_idx;
  }
  double mv[4][4] = {{0}};
  double mi[4][4] = {{0}};
  const int64_t chunk = 4 * L;
  const int64_t n_chunks = n / chunk;
  for (int64_t c = 0; c < n_chunks; c++) {
    const double *xp = x + c * chunk;
    for (int acc = 0; acc < 4; acc++) {
      for (int l = 0; l < L; l++) {
        double v = fabs(xp[acc * L + l]);
        if (v > mv[acc][l]) {
          mv[acc][l] = v;
          mi[acc][l] = (double)(c * chunk + acc * L + l);
        }
      }
    }
  }
  for (int acc = 1; acc < 4; acc++) {
    for (int l = 0; l < L; l++) {
      if (mv[acc][l] > mv[0][l]) {
        mv[0][l] = mv[acc][l];
        mi[0][l] = mi[acc][l];
      }
    }
  }
  double max_val = mv[0][0];
  int64_t max_idx = (int64_t)mi[0][0];
  for (int l = 1; l < L; l++) {
    if (mv[0][l] > max_val) {
      max_val = mv[0][l];
      max_idx = (int64_t)mi[0][l];
    }
  }
  for (int64_t i = n_chunks * chunk; i < n; i++) {
    double v = fabs(x[i]);
    if (v > max_val) {
      max_val = v;
      max_idx = i;
    }
  }
  return max_idx;
}

/* src/scal.rs:6-22 / :24-40: vector multiply over whole chunks, returns the
 * count processed; the caller finishes the tail with the same multiply. */
int64_t oracle_scal_kernel(int64_t m, double inv_diag, double *col) {
  const int64_t done = (m / g_lanes) * g_lanes;
  for (int64_t i = 0; i < done; i++) col[i] = col[i] * inv_diag;
  return done;
}

/* src/scal.rs:45-57 */
void oracle_scal(int64_t n, double alpha, double *x, int64_t incx) {
  if (incx == 1) {
    int64_t p = oracle_scal_kernel(n, alpha, x);
    for (int64_t i = p; i < n; i++) x[i] *= alpha;
  } else {
    for (int64_t i = 0; i < n; i++) x[i * incx] *= alpha;
  }
}

/* src/ger.rs:28-61 with the kernel :63-90 / :92-119.  Column pairs whose two
 * scale factors are both zero are skipped; the vector body is fused, the row
 * tail and the odd last column are not. */
void oracle_ger(int64_t m, int64_t n, double alpha, const double *x, const double *y, int64_t ldy,
                double *a, int64_t lda) {
  const int64_t n_unrolled = n - (n % 2);
  const int64_t rows_vec = (m / g_lanes) * g_lanes;
  for (int64_t j = 0; j < n_unrolled; j += 2) {
    const double t0 = alpha * y[j * ldy];
    const double t1 = alpha * y[(j + 1) * ldy];
    if (t0 == 0.0 && t1 == 0.0) continue;
    double *a0 = a + j * lda;
    double *a1 = a + (j + 1) * lda;
    for (int64_t i = 0; i < rows_vec; i++) {
      a0[i] = ORACLE_FMA(x[i], t0, a0[i]);
      a1[i] = ORACLE_FMA(x[i], t1, a1[i]);
    }
    for (int64_t i = rows_vec; i < m; i++) {
      a0[i] += t0 * x[i];
      a1[i] += t1 * x[i];
    }
  }
  if (n % 2 != 0) {
    const int64_t j = n - 1;
    const double t = alpha * y[j * ldy];
    if (t != 0.0) {
      for (int64_t i = 0; i < m; i++) a[i + j * lda] += t * x[i];
    }
  }
}

/* src/utilities.rs:18-54 (AVX2) / :58-92 (NEON). */
double oracle_dot_product(int64_t n, const double *x, int64_t incx, const double *y, int64_t incy) {
  if (n == 0) return 0.0;
  if (incx == 1 && incy == 1) {
    const int L = g_lanes;
    const int64_t n_chunks = n / L;
    double lane[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = 0; i < n_chunks; i++)
      for (int l = 0; l < L; l++) lane[l] = ORACLE_FMA(x[i * L + l], y[i * L + l], lane[l]);
    double s;
    if (L == 4) {
      /* temp_sum = 0.0; temp_sum += lanes.iter().sum() */
      double h = -0.0;
      for (int l = 0; l < 4; l++) h = h + lane[l];
      s = 0.0;
      s += h;
    } else {
      s = lane[0] + lane[1]; /* vaddvq_f64 */
    }
    for (int64_t i = n_chunks * L; i < n; i++) s += x[i] * y[i];
    return s;
  }
  double s = 0.0;
  for (int64_t i = 0; i < n; i++) s += x[i * incx] * y[i * incy];
  return s;
}

/* src/utilities.rs:103-132 (AVX2) / :136-164 (NEON). */
void oracle_daxpy(int64_t n, double alpha, const double *x, int64_t incx, double *y, int64_t incy) {
  if (n == 0 || alpha == 0.0) return;
  if (incx == 1 && incy == 1) {
    const int64_t done = (n / g_lanes) * g_lanes;
    for (int64_t i = 0; i < done; i++) y[i] = ORACLE_FMA(alpha, x[i], y[i]);
    for (int64_t i = done; i < n; i++) y[i] += alpha * x[i];
  } else {
    for (int64_t i = 0; i < n; i++) y[i * incy] += alpha * x[i * incx];
  }
}

/* ------------------------------------------------------------------------ */
/* GEMM: src/gemm.rs                                                          */
/* ------------------------------------------------------------------------ */
enum { KC = 64, MC = 32, NC = 16, MR = 8, NR = 4, GEMM_PAR = 128 };

/* src/gemm.rs:49-65; the 'N' test is case-sensitive, as in BOLA. */
static void pack(char trans, int64_t rows, int64_t cols, const double *src, int64_t ld, double *dst) {
  if (trans == 'N') {
    for (int64_t j = 0; j < cols; j++)
      for (int64_t i = 0; i < rows; i++) dst[i + j * rows] = src[i + j * ld];
  } else {
    for (int64_t j = 0; j < cols; j++)
      for (int64_t i = 0; i < rows; i++) dst[i + j * rows] = src[j + i * ld];
  }
}

/* src/gemm.rs:228-270 / :274-336: an 8x4 block accumulated from zero with
 * FMA over the K chunk, then C = fma(alpha, acc, C). */
static void add_8x4_kernel(int64_t k, double alpha, const double *a, int64_t lda, const double *b,
                           int64_t ldb, double *c, int64_t ldc) {
  double acc[NR][MR];
  for (int j = 0; j < NR; j++)
    for (int i = 0; i < MR; i++) acc[j][i] = 0.0;
  for (int64_t l = 0; l < k; l++) {
    const double *al = a + l * lda;
    for (int j = 0; j < NR; j++) {
      const double bj = b[l + j * ldb];
      for (int i = 0; i < MR; i++) acc[j][i] = ORACLE_FMA(al[i], bj, acc[j][i]);
    }
  }
  for (int j = 0; j < NR; j++) {
    double *cp = c + j * ldc;
    for (int i = 0; i < MR; i++) cp[i] = ORACLE_FMA(alpha, acc[j][i], cp[i]);
  }
}

/* src/gemm.rs:357-377: unfused c += (alpha*b) * a for edge blocks. */
static void add_scalar_kernel(int64_t m, int64_t n, int64_t k, double alpha, const double *a,
                              int64_t lda, const double *b, int64_t ldb, double *c, int64_t ldc) {
  for (int64_t j = 0; j < n; j++) {
    for (int64_t l = 0; l < k; l++) {
      const double temp = alpha * b[l + j * ldb];
      for (int64_t i = 0; i < m; i++) c[i + j * ldc] += temp * a[i + l * lda];
    }
  }
}

/* src/gemm.rs:152-216: one NC-wide column block of C. */
static void gemm_block(int64_t jc, char transa, char transb, int notransa, int notransb, int64_t m,
                       int64_t n, int64_t k, double alpha, const double *a, int64_t lda,
                       const double *b, int64_t ldb, double *c, int64_t ldc) {
  double a_packed[MC * KC];
  double b_packed[KC * NC];
  const int64_t nb = imin(n - jc, NC);
  for (int64_t pc = 0; pc < k; pc += KC) {
    const int64_t pb = imin(k - pc, KC);
    const double *bp = notransb ? b + pc + jc * ldb : b + jc + pc * ldb;
    pack(transb, pb, nb, bp, ldb, b_packed);
    for (int64_t ic = 0; ic < m; ic += MC) {
      const int64_t mb = imin(m - ic, MC);
      const double *ap = notransa ? a + ic + pc * lda : a + pc + ic * lda;
      pack(transa, mb, pb, ap, lda, a_packed);
      for (int64_t j = 0; j < nb; j += NR) {
        for (int64_t i = 0; i < mb; i += MR) {
          double *cb = c + ic + i + (jc + j) * ldc;
          const double *bpk = b_packed + j * pb;
          if (i + MR > mb || j + NR > nb) {
            add_scalar_kernel(imin(mb - i, MR), imin(nb - j, NR), pb, alpha, a_packed + i, mb, bpk,
                              pb, cb, ldc);
          } else {
            add_8x4_kernel(pb, alpha, a_packed + i, mb, bpk, pb, cb, ldc);
          }
        }
      }
    }
  }
}

/* src/gemm.rs:103-226 */
void oracle_gemm(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
                 const double *a, int64_t lda, const double *b, int64_t ldb, double beta,
                 double *c, int64_t ldc) {
  if (m == 0 || n == 0) return;
  if (beta == 0.0) {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < m; i++) c[i + j * ldc] = 0.0;
  } else if (beta != 1.0) {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < m; i++) c[i + j * ldc] *= beta;
  }
  if (alpha == 0.0) return;
  const int notransa = is_ch(transa, 'N');
  const int notransb = is_ch(transb, 'N');
  const int64_t nblocks = (n + NC - 1) / NC;
  if (n > GEMM_PAR) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(oracle_get_threads())
    for (int64_t bi = 0; bi < nblocks; bi++)
      gemm_block(bi * NC, transa, transb, notransa, notransb, m, n, k, alpha, a, lda, b, ldb, c, ldc);
  } else {
    for (int64_t bi = 0; bi < nblocks; bi++)
      gemm_block(bi * NC, transa, transb, notransa, notransb, m, n, k, alpha, a, lda, b, ldb, c, ldc);
  }
}

/* ------------------------------------------------------------------------ */
/* TRSM: src/trsm.rs                                                          */
/* ------------------------------------------------------------------------ */
enum { TRSM_STOP = 64, TRSM_PAR = 32 };

/* src/trsm.rs:96-109 (base case of trsm_lnl) for one column. */
static void lnl_col(int unit, int64_t m, const double *a, int64_t lda, double *bc) {
  for (int64_t k = 0; k < m; k++) {
    const double bkj = bc[k];
    if (bkj != 0.0) {
      const double u = unit ? bkj : bkj / a[k + k * lda];
      bc[k] = u;
      if (m > k + 1) oracle_daxpy(m - k - 1, -u, a + k + 1 + k * lda, 1, bc + k + 1, 1);
    }
  }
}
/* src/trsm.rs:137-149 */
static void lnu_col(int unit, int64_t m, const double *a, int64_t lda, double *bc) {
  for (int64_t k = m - 1; k >= 0; k--) {
    const double bkj = bc[k];
    if (bkj != 0.0) {
      const double u = unit ? bkj : bkj / a[k + k * lda];
      bc[k] = u;
      if (k > 0) oracle_daxpy(k, -u, a + k * lda, 1, bc, 1);
    }
  }
}
/* src/trsm.rs:176-188 */
static void ltl_col(int unit, int64_t m, const double *a, int64_t lda, double *bc) {
  for (int64_t i = m - 1; i >= 0; i--) {
    double t = bc[i];
    for (int64_t k = i + 1; k < m; k++) t -= a[k + i * lda] * bc[k];
    if (!unit) t /= a[i + i * lda];
    bc[i] = t;
  }
}
/* src/trsm.rs:215-227 */
static void ltu_col(int unit, int64_t m, const double *a, int64_t lda, double *bc) {
  for (int64_t i = 0; i < m; i++) {
    double t = bc[i];
    for (int64_t k = 0; k < i; k++) t -= a[k + i * lda] * bc[k];
    if (!unit) t /= a[i + i * lda];
    bc[i] = t;
  }
}

typedef void (*col_fn)(int, int64_t, const double *, int64_t, double *);

static void left_base(col_fn f, int unit, int64_t m, int64_t n, const double *a, int64_t lda,
                      double *b, int64_t ldb) {
  if (n > TRSM_PAR) {
#pragma omp parallel for schedule(static) num_threads(oracle_get_threads())
    for (int64_t j = 0; j < n; j++) f(unit, m, a, lda, b + j * ldb);
  } else {
    for (int64_t j = 0; j < n; j++) f(unit, m, a, lda, b + j * ldb);
  }
}

/* src/trsm.rs:95-131 */
static void trsm_lnl(int unit, int64_t m, int64_t n, const double *a, int64_t lda, double *b,
                     int64_t ldb) {
  if (m <= TRSM_STOP) {
    left_base(lnl_col, unit, m, n, a, lda, b, ldb);
    return;
  }
  const int64_t m1 = m / 2, m2 = m - m1;
  trsm_lnl(unit, m1, n, a, lda, b, ldb);
  oracle_gemm('N', 'N', m2, n, m1, -1.0, a + m1, lda, b, ldb, 1.0, b + m1, ldb);
  trsm_lnl(unit, m2, n, a + m1 + m1 * lda, lda, b + m1, ldb);
}
/* src/trsm.rs:135-170 */
static void trsm_lnu(int unit, int64_t m, int64_t n, const double *a, int64_t lda, double *b,
                     int64_t ldb) {
  if (m <= TRSM_STOP) {
    left_base(lnu_col, unit, m, n, a, lda, b, ldb);
    return;
  }
  const int64_t m1 = m / 2, m2 = m - m1;
  trsm_lnu(unit, m2, n, a + m1 + m1 * lda, lda, b + m1, ldb);
  oracle_gemm('N', 'N', m1, n, m2, -1.0, a + m1 * lda, lda, b + m1, ldb, 1.0, b, ldb);
  trsm_lnu(unit, m1, n, a, lda, b, ldb);
}
/* src/trsm.rs:174-209 */
static void trsm_ltl(int unit, int64_t m, int64_t n, const double *a, int64_t lda, double *b,
                     int64_t ldb) {
  if (m <= TRSM_STOP) {
    left_base(ltl_col, unit, m, n, a, lda, b, ldb);
    return;
  }
  const int64_t m1 = m / 2, m2 = m - m1;
  trsm_ltl(unit, m2, n, a + m1 + m1 * lda, lda, b + m1, ldb);
  oracle_gemm('T', 'N', m1, n, m2, -1.0, a + m1, lda, b + m1, ldb, 1.0, b, ldb);
  trsm_ltl(unit, m1, n, a, lda, b, ldb);
}
/* src/trsm.rs:213-248 */
static void trsm_ltu(int unit, int64_t m, int64_t n, const double *a, int64_t lda, double *b,
                     int64_t ldb) {
  if (m <= TRSM_STOP) {
    left_base(ltu_col, unit, m, n, a, lda, b, ldb);
    return;
  }
  const int64_t m1 = m / 2, m2 = m - m1;
  trsm_ltu(unit, m1, n, a, lda, b, ldb);
  oracle_gemm('T', 'N', m2, n, m1, -1.0, a + m1 * lda, lda, b, ldb, 1.0, b + m1, ldb);
  trsm_ltu(unit, m2, n, a + m1 + m1 * lda, lda, b + m1, ldb);
}

static void scale_col_recip(int unit, int64_t m, const double *a, int64_t lda, int64_t j, double *bj) {
  if (!unit) {
    const double inv = 1.0 / a[j + j * lda];
    for (int64_t i = 0; i < m; i++) bj[i] *= inv;
  }
}

/* src/trsm.rs:252-280 */
static void trsm_rnl(int unit, int64_t m, int64_t n, const double *a, int64_t lda, double *b,
                     int64_t ldb) {
  if (n <= TRSM_STOP) {
    for (int64_t j = n - 1; j >= 0; j--) {
      double *bj = b + j * ldb;
      for (int64_t k = j + 1; k < n; k++) {
        const double akj = a[k + j * lda];
        if (akj != 0.0) {
          const double *bk = b + k * ldb;
          for (int64_t i = 0; i < m; i++) bj[i] -= akj * bk[i];
        }
      }
      scale_col_recip(unit, m, a, lda, j, bj);
    }
    return;
  }
  const int64_t n1 = n / 2, n2 = n - n1;
  trsm_rnl(unit, m, n2, a + n1 + n1 * lda, lda, b + n1 * ldb, ldb);
  oracle_gemm('N', 'N', m, n1, n2, -1.0, b + n1 * ldb, ldb, a + n1, lda, 1.0, b, ldb);
  trsm_rnl(unit, m, n1, a, lda, b, ldb);
}
/* src/trsm.rs:284-312 */
static void trsm_rnu(int unit, int64_t m, int64_t n, const double *a, int64_t lda, double *b,
                     int64_t ldb) {
  if (n <= TRSM_STOP) {
    for (int64_t j = 0; j < n; j++) {
      double *bj = b + j * ldb;
      for (int64_t k = 0; k < j; k++) {
        const double akj = a[k + j * lda];
        if (akj != 0.0) {
          const double *bk = b + k * ldb;
          for (int64_t i = 0; i < m; i++) bj[i] -= akj * bk[i];
        }
      }
      scale_col_recip(unit, m, a, lda, j, bj);
    }
    return;
  }
  const int64_t n1 = n / 2, n2 = n - n1;
  trsm_rnu(unit, m, n1, a, lda, b, ldb);
  oracle_gemm('N', 'N', m, n2, n1, -1.0, b, ldb, a + n1 * lda, lda, 1.0, b + n1 * ldb, ldb);
  trsm_rnu(unit, m, n2, a + n1 + n1 * lda, lda, b + n1 * ldb, ldb);
}
/* src/trsm.rs:316-344 */
static void trsm_rtl(int unit, int64_t m, int64_t n, const double *a, int64_t lda, double *b,
                     int64_t ldb) {
  if (n <= TRSM_STOP) {
    for (int64_t j = 0; j < n; j++) {
      double *bj = b + j * ldb;
      for (int64_t k = 0; k < j; k++) {
        const double ajk = a[j + k * lda];
        if (ajk != 0.0) {
          const double *bk = b + k * ldb;
          for (int64_t i = 0; i < m; i++) bj[i] -= ajk * bk[i];
        }
      }
      scale_col_recip(unit, m, a, lda, j, bj);
    }
    return;
  }
  const int64_t n1 = n / 2, n2 = n - n1;
  trsm_rtl(unit, m, n1, a, lda, b, ldb);
  oracle_gemm('N', 'T', m, n2, n1, -1.0, b, ldb, a + n1, lda, 1.0, b + n1 * ldb, ldb);
  trsm_rtl(unit, m, n2, a + n1 + n1 * lda, lda, b + n1 * ldb, ldb);
}
/* src/trsm.rs:348-376 */
static void trsm_rtu(int unit, int64_t m, int64_t n, const double *a, int64_t lda, double *b,
                     int64_t ldb) {
  if (n <= TRSM_STOP) {
    for (int64_t j = n - 1; j >= 0; j--) {
      double *bj = b + j * ldb;
      for (int64_t k = j + 1; k < n; k++) {
        const double ajk = a[j + k * lda];
        if (ajk != 0.0) {
          const double *bk = b + k * ldb;
          for (int64_t i = 0; i < m; i++) bj[i] -= ajk * bk[i];
        }
      }
      scale_col_recip(unit, m, a, lda, j, bj);
    }
    return;
  }
  const int64_t n1 = n / 2, n2 = n - n1;
  trsm_rtu(unit, m, n2, a + n1 + n1 * lda, lda, b + n1 * ldb, ldb);
  oracle_gemm('N', 'T', m, n1, n2, -1.0, b + n1 * ldb, ldb, a + n1 * lda, lda, 1.0, b, ldb);
  trsm_rtu(unit, m, n1, a, lda, b, ldb);
}

/* src/trsm.rs:33-91: alpha pre-scale, then case-insensitive dispatch. */
void oracle_trsm(char side, char uplo, char transa, char diag, int64_t m, int64_t n, double alpha,
                 const double *a, int64_t lda, double *b, int64_t ldb) {
  if (m == 0 || n == 0) return;
  if (alpha != 1.0) {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < m; i++) b[i + j * ldb] *= alpha;
  }
  const int lside = is_ch(side, 'L');
  const int upper = is_ch(uplo, 'U');
  const int notrans = is_ch(transa, 'N');
  const int unit = is_ch(diag, 'U');
  if (lside) {
    if (notrans) {
      if (upper) trsm_lnu(unit, m, n, a, lda, b, ldb);
      else trsm_lnl(unit, m, n, a, lda, b, ldb);
    } else if (upper) {
      trsm_ltu(unit, m, n, a, lda, b, ldb);
    } else {
      trsm_ltl(unit, m, n, a, lda, b, ldb);
    }
  } else if (notrans) {
    if (upper) trsm_rnu(unit, m, n, a, lda, b, ldb);
    else trsm_rnl(unit, m, n, a, lda, b, ldb);
  } else if (upper) {
    trsm_rtu(unit, m, n, a, lda, b, ldb);
  } else {
    trsm_rtl(unit, m, n, a, lda, b, ldb);
  }
}

/* ------------------------------------------------------------------------ */
/* SYRK: src/syrk.rs (restated with its diagonal-block addressing, which is    */
/* wrong for (U,N) and (L,T) once n > 32 or k > 32)                           */
/* ------------------------------------------------------------------------ */
enum { SYRK_NB = 32 };

/* src/syrk.rs:190-249 */
static void syrk_kernel(char uplo, char trans, int64_t n, int64_t k, double alpha, const double *a,
                        int64_t lda, double *c, int64_t ldc, char original_trans) {
  if (trans == 'N') {
    if (uplo == 'U') {
      for (int64_t j = 0; j < n; j++)
        for (int64_t l = 0; l < k; l++) {
          const double t = alpha * a[j + l * lda];
          if (t != 0.0) oracle_daxpy(j + 1, t, a + l * lda, 1, c + j * ldc, 1);
        }
    } else {
      for (int64_t j = 0; j < n; j++)
        for (int64_t l = 0; l < k; l++) {
          const double t = alpha * a[j + l * lda];
          if (t != 0.0) oracle_daxpy(n - j, t, a + j + l * lda, 1, c + j + j * ldc, 1);
        }
    }
  } else {
    const int ot = (original_trans == 'T');
    const int64_t s = ot ? 1 : lda;
    for (int64_t j = 0; j < n; j++) {
      const int64_t i0 = (uplo == 'U') ? 0 : j;
      const int64_t i1 = (uplo == 'U') ? j + 1 : n;
      for (int64_t i = i0; i < i1; i++) {
        const double *ri = ot ? a + i * lda : a + i;
        const double *rj = ot ? a + j * lda : a + j;
        const double t = oracle_dot_product(k, ri, s, rj, s);
        c[i + j * ldc] += alpha * t;
      }
    }
  }
}

/* src/syrk.rs:17-186 */
void oracle_syrk(char uplo, char trans, int64_t n, int64_t k, double alpha, const double *a,
                 int64_t lda, double beta, double *c, int64_t ldc) {
  if (n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return;
  if (beta == 0.0 || beta != 1.0) {
    for (int64_t j = 0; j < n; j++) {
      const int64_t i0 = (uplo == 'U') ? 0 : j;
      const int64_t i1 = (uplo == 'U') ? j + 1 : n;
      for (int64_t i = i0; i < i1; i++) {
        if (beta == 0.0) c[i + j * ldc] = 0.0;
        else c[i + j * ldc] *= beta;
      }
    }
  }
  if (alpha == 0.0) return;
  if (uplo == 'U') {
    for (int64_t j = 0; j < n; j += SYRK_NB) {
      const int64_t jb = imin(n - j, SYRK_NB);
      for (int64_t p = 0; p < k; p += SYRK_NB) {
        const int64_t pb = imin(k - p, SYRK_NB);
        syrk_kernel('U', trans, jb, pb, alpha, a + j * lda + p, lda, c + j + j * ldc, ldc, trans);
        for (int64_t i = 0; i < j; i += SYRK_NB) {
          const int64_t ib = imin(j - i, SYRK_NB);
          if (trans == 'T')
            oracle_gemm('T', 'N', ib, jb, pb, alpha, a + p + i * lda, lda, a + p + j * lda, lda, 1.0,
                        c + i + j * ldc, ldc);
          else
            oracle_gemm('N', 'T', ib, jb, pb, alpha, a + i + p * lda, lda, a + j + p * lda, lda, 1.0,
                        c + i + j * ldc, ldc);
        }
      }
    }
  } else {
    for (int64_t j = 0; j < n; j += SYRK_NB) {
      const int64_t jb = imin(n - j, SYRK_NB);
      for (int64_t p = 0; p < k; p += SYRK_NB) {
        const int64_t pb = imin(k - p, SYRK_NB);
        syrk_kernel('L', trans, jb, pb, alpha, a + j + p * lda, lda, c + j + j * ldc, ldc, trans);
        for (int64_t i = j + jb; i < n; i += SYRK_NB) {
          const int64_t ib = imin(n - i, SYRK_NB);
          if (trans == 'N')
            oracle_gemm('N', 'T', ib, jb, pb, alpha, a + i + p * lda, lda, a + j + p * lda, lda, 1.0,
                        c + i + j * ldc, ldc);
          else
            oracle_gemm('T', 'N', ib, jb, pb, alpha, a + p + i * lda, lda, a + p + j * lda, lda, 1.0,
                        c + i + j * ldc, ldc);
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* LASWP: src/laswp.rs:22-132                                                 */
/* ------------------------------------------------------------------------ */
enum { LASWP_PAR = 256 };

static void laswp_cols(int64_t c0, int64_t c1, double *a, int64_t lda, int64_t ix0, int32_t i1,
                       int32_t i2, int32_t i_inc, const int32_t *ipiv, int32_t incx) {
  for (int64_t col = c0; col < c1; col++) {
    double *cp = a + col * lda;
    int64_t ix = ix0;
    int32_t i = i1;
    while (i_inc > 0 ? i <= i2 : i >= i2) {
      const int64_t ip = ipiv[ix];
      if (ip != (int64_t)i) {
        const double t = cp[i - 1];
        cp[i - 1] = cp[ip - 1];
        cp[ip - 1] = t;
      }
      ix += incx;
      i += i_inc;
    }
  }
}

void oracle_laswp(int64_t n, double *a, int64_t lda, int32_t k1, int32_t k2, const int32_t *ipiv,
                  int32_t incx) {
  if (n == 0 || incx == 0 || k1 > k2) return;
  int64_t ix0;
  int32_t i1, i2, i_inc;
  if (incx > 0) {
    ix0 = k1 - 1;
    i1 = k1;
    i2 = k2;
    i_inc = 1;
  } else {
    ix0 = (int64_t)(k1 - 1) + (int64_t)(k2 - k1) * (int64_t)(-(int64_t)incx);
    i1 = k2;
    i2 = k1;
    i_inc = -1;
  }
  /* Every column sees the same sequence of swaps, so the column split of the
   * serial (4-column unroll) and parallel (32-column chunk) forms does not
   * change any result. */
  if (n < LASWP_PAR) {
    laswp_cols(0, n, a, lda, ix0, i1, i2, i_inc, ipiv, incx);
    return;
  }
  const int64_t n32 = (n / 32) * 32;
  const int64_t nchunks = n32 / 32;
#pragma omp parallel for schedule(static) num_threads(oracle_get_threads())
  for (int64_t cidx = 0; cidx < nchunks; cidx++)
    laswp_cols(cidx * 32, cidx * 32 + 32, a, lda, ix0, i1, i2, i_inc, ipiv, incx);
  if (n32 != n) laswp_cols(n32, n, a, lda, ix0, i1, i2, i_inc, ipiv, incx);
}

/* ------------------------------------------------------------------------ */
/* GETRF: src/getrf.rs, src/getrf2.rs                                         */
/* ------------------------------------------------------------------------ */
enum { GETRF_NB = 32, RECURSION_STOP = 32 };

static void record_margin(int64_t col, int64_t len, const double *x) {
  if (!g_margins || col < 0 || col >= g_margins_len) return;
  double m1 = -1.0, m2 = -1.0;
  for (int64_t i = 0; i < len; i++) {
    const double v = fabs(x[i]);
    if (v > m1) {
      m2 = m1;
      m1 = v;
    } else if (v > m2) {
      m2 = v;
    }
  }
  g_margins[col] = (m1 > 0.0 && m2 >= 0.0) ? (m1 - m2) / m1 : 1.0;
}

/* src/getrf2.rs:131-185: unblocked LU of an m x n panel.  Returns 0 or the
 * 1-based column (local to this panel) whose pivot is exactly zero. */
static int iterative_getrf2(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv,
                            int64_t col_offset) {
  const int64_t min_mn = imin(m, n);
  for (int64_t j = 0; j < min_mn; j++) {
    if (g_margins) record_margin(col_offset + j, m - j, a + j + j * lda);
    const int64_t jp = j + oracle_idamax(m - j, a + j + j * lda);
    ipiv[j] = (int32_t)(jp + 1);
    if (a[jp + j * lda] != 0.0) {
      if (jp != j) {
        for (int64_t k = 0; k < n; k++) {
          const double t = a[j + k * lda];
          a[j + k * lda] = a[jp + k * lda];
          a[jp + k * lda] = t;
        }
      }
      if (j < m - 1) {
        const double ajj = a[j + j * lda];
        const double inv = 1.0 / ajj;
        const int64_t m_rem = m - (j + 1);
        double *col = a + j + 1 + j * lda;
        const int64_t p = oracle_scal_kernel(m_rem, inv, col);
        for (int64_t i = p; i < m_rem; i++) col[i] *= inv;
      }
    } else {
      return (int)(j + 1);
    }
    if (j < min_mn - 1) {
      oracle_ger(m - j - 1, n - j - 1, -1.0, a + j + 1 + j * lda, a + j + (j + 1) * lda, lda,
                 a + j + 1 + (j + 1) * lda, lda);
    }
  }
  return 0;
}

/* src/getrf2.rs:39-106 (recursive; returns global 1-based column on a zero pivot). */
static int getrf2_at(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv, int64_t col_offset) {
  if (lda < imax(m, 1)) return -4;
  if (m == 0 || n == 0) return 0;
  if (m <= RECURSION_STOP || n <= RECURSION_STOP) return iterative_getrf2(m, n, a, lda, ipiv, col_offset);
  const int64_t n1 = imin(m, n) / 2;
  const int64_t n2 = n - n1;
  int r = getrf2_at(m, n1, a, lda, ipiv, col_offset);
  if (r) return r;
  oracle_laswp(n2, a + n1 * lda, lda, 1, (int32_t)n1, ipiv, 1);
  oracle_trsm('L', 'L', 'N', 'U', n1, n2, 1.0, a, lda, a + n1 * lda, lda);
  if (n1 < m)
    oracle_gemm('N', 'N', m - n1, n2, n1, -1.0, a + n1, lda, a + n1 * lda, lda, 1.0,
                a + n1 + n1 * lda, lda);
  if (n1 < m) {
    r = getrf2_at(m - n1, n2, a + n1 + n1 * lda, lda, ipiv + n1, col_offset + n1);
    if (r) return r > 0 ? r + (int)n1 : r;
  }
  for (int64_t i = n1; i < imin(m, n); i++) ipiv[i] += (int32_t)n1;
  oracle_laswp(n1, a, lda, (int32_t)(n1 + 1), (int32_t)imin(m, n), ipiv, 1);
  return 0;
}

int oracle_getrf2(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv) {
  return getrf2_at(m, n, a, lda, ipiv, 0);
}

/* src/getrf.rs:37-101 */
int oracle_getrf(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv) {
  if (lda < imax(m, 1)) return -4;
  if (m == 0 || n == 0) return 0;
  const int64_t min_mn = imin(m, n);
  if (GETRF_NB >= min_mn) return getrf2_at(m, n, a, lda, ipiv, 0);
  for (int64_t j = 0; j < min_mn; j += GETRF_NB) {
    const int64_t jb = imin(GETRF_NB, min_mn - j);
    int r = getrf2_at(m - j, jb, a + j + j * lda, lda, ipiv + j, j);
    if (r) return r > 0 ? r + (int)j : r;
    for (int64_t i = j; i < j + jb; i++) ipiv[i] += (int32_t)j;
    const int32_t k1 = (int32_t)(j + 1), k2 = (int32_t)(j + jb);
    if (j > 0) oracle_laswp(j, a, lda, k1, k2, ipiv, 1);
    if (j + jb < n) {
      oracle_laswp(n - j - jb, a + (j + jb) * lda, lda, k1, k2, ipiv, 1);
      const double *l11 = a + j + j * lda;
      double *u12 = a + j + (j + jb) * lda;
      oracle_trsm('L', 'L', 'N', 'U', jb, n - j - jb, 1.0, l11, lda, u12, lda);
      if (j + jb < m)
        oracle_gemm('N', 'N', m - j - jb, n - j - jb, jb, -1.0, a + (j + jb) + j * lda, lda, u12, lda,
                    1.0, a + (j + jb) + (j + jb) * lda, lda);
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* POTRF: src/potrf.rs, src/potrf2.rs                                         */
/* ------------------------------------------------------------------------ */
enum { POTRF_NB = 32 };

/* src/potrf2.rs:36-80 (returns 0 or the 1-based failing column). */
static int potrf2_rec(char uplo, int64_t n, double *a, int64_t lda) {
  if (n == 0) return 0;
  if (n == 1) {
    const double a11 = a[0];
    if (a11 > 0.0) {
      a[0] = sqrt(a11);
      return 0;
    }
    return 1;
  }
  const int64_t n1 = n / 2, n2 = n - n1;
  int r = potrf2_rec(uplo, n1, a, lda);
  if (r) return r;
  double *a22 = a + n1 + n1 * lda;
  if (uplo == 'U') {
    double *a12 = a + n1 * lda;
    oracle_trsm('L', 'U', 'T', 'N', n1, n2, 1.0, a, lda, a12, lda);
    oracle_syrk('U', 'T', n2, n1, -1.0, a12, lda, 1.0, a22, lda);
  } else {
    double *a21 = a + n1;
    oracle_trsm('R', 'L', 'T', 'N', n2, n1, 1.0, a, lda, a21, lda);
    oracle_syrk('L', 'N', n2, n1, -1.0, a21, lda, 1.0, a22, lda);
  }
  r = potrf2_rec(uplo, n2, a22, lda);
  if (r) return r + (int)n1;
  return 0;
}

int oracle_potrf2(char uplo, int64_t n, double *a, int64_t lda) { return potrf2_rec(uplo, n, a, lda); }

/* src/potrf.rs:101-181 (left-looking, NB = 32); failing column is global. */
int oracle_potrf(char uplo, int64_t n, double *a, int64_t lda) {
  if (uplo != 'U' && uplo != 'L') return -1;
  if (lda < imax(n, 1)) return -4;
  if (POTRF_NB >= n) return potrf2_rec(uplo, n, a, lda);
  for (int64_t j = 0; j < n; j += POTRF_NB) {
    const int64_t jb = imin(POTRF_NB, n - j);
    double *ajj = a + j + j * lda;
    if (uplo == 'U') {
      double *a1j = a + j * lda;
      oracle_syrk('U', 'T', jb, j, -1.0, a1j, lda, 1.0, ajj, lda);
      int r = potrf2_rec('U', jb, ajj, lda);
      if (r) return r + (int)j;
      if (j + jb < n) {
        const int64_t n_rem = n - j - jb;
        oracle_gemm('T', 'N', jb, n_rem, j, -1.0, a1j, lda, a + (j + jb) * lda, lda, 1.0,
                    a + j + (j + jb) * lda, lda);
        oracle_trsm('L', 'U', 'T', 'N', jb, n_rem, 1.0, ajj, lda, a + j + (j + jb) * lda, lda);
      }
    } else {
      double *aj0 = a + j;
      oracle_syrk('L', 'N', jb, j, -1.0, aj0, lda, 1.0, ajj, lda);
      int r = potrf2_rec('L', jb, ajj, lda);
      if (r) return r + (int)j;
      if (j + jb < n) {
        const int64_t n_rem = n - j - jb;
        oracle_gemm('N', 'T', n_rem, jb, j, -1.0, a + j + jb, lda, aj0, lda, 1.0,
                    a + j + jb + j * lda, lda);
        oracle_trsm('R', 'L', 'T', 'N', n_rem, jb, 1.0, ajj, lda, a + j + jb + j * lda, lda);
      }
    }
  }
  return 0;
}
