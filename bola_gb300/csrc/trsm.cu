// trsm.cu — triangular solves with BOLA's recursion and rounding
// (src/trsm.rs:33-376).
//
// The host walks BOLA's recursion (halving down to 64) and issues the exact
// DGEMM for every off-diagonal block, so >97% of the flops run in the GEMM
// kernel.  The <=64 base cases run on the GPU with BOLA's per-element order:
//   left, no transpose  — column forward/back substitution with BOLA's daxpy
//                         (a warp per right-hand side, rows across lanes);
//   left, transpose     — dot-style substitution, one thread per column;
//   right               — column sweeps, one thread per row of B.
#include "common.cuh"

namespace bola {
namespace {

constexpr int STOP = 64;  // TRSM_RECURSION_STOP (src/trsm.rs:8)

__global__ void scale_matrix(int64_t m, int64_t n, double alpha, double *B, int64_t ldb,
                             const int32_t *info) {
  if (stop_flag(info)) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * n) return;
  const int64_t i = e % m, j = e / m;
  B[i + j * ldb] = __dmul_rn(B[i + j * ldb], alpha);
}

// Loads the m x m triangle block (column-major, ld = STOP) into shared memory.
__device__ __forceinline__ void load_tri(double *sA, const double *A, int64_t lda, int m) {
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int i = e % m, k = e / m;
    sA[i + k * STOP] = A[i + (int64_t)k * lda];
  }
}

// Left side, op(A) = A: trsm_lnl / trsm_lnu base cases (src/trsm.rs:96-123, 136-163).
template <bool LOWER>
__global__ void __launch_bounds__(256)
left_n_base(int m, int64_t n, bool unit, const double *__restrict__ A, int64_t lda, double *B,
            int64_t ldb, int lanes, const int32_t *info) {
  __shared__ double sA[STOP * STOP];
  if (stop_flag(info)) return;
  load_tri(sA, A, lda, m);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t col = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (col >= n) return;
  double *bc = B + col * ldb;
  double b0 = lane < m ? bc[lane] : 0.0;
  double b1 = lane + 32 < m ? bc[lane + 32] : 0.0;
  for (int step = 0; step < m; ++step) {
    const int k = LOWER ? step : m - 1 - step;
    const double bk = __shfl_sync(0xffffffffu, k < 32 ? b0 : b1, k & 31);
    if (bk == 0.0) continue;  // BOLA skips zero entries (src/trsm.rs:101,141)
    const double u = unit ? bk : bk / sA[k + k * STOP];
    if (k == lane) b0 = u;
    if (k == lane + 32) b1 = u;
    if (u == 0.0) continue;  // daxpy returns early for a zero scale (src/utilities.rs:108)
    // daxpy over rows k+1..m-1 (lower) or 0..k-1 (upper) with alpha = -u
    const int64_t len = LOWER ? (int64_t)(m - k - 1) : (int64_t)k;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = lane + 32 * h;
      const bool in = LOWER ? (i > k && i < m) : (i < k);
      if (!in) continue;
      const int64_t idx = LOWER ? (int64_t)(i - k - 1) : (int64_t)i;
      double &bi = h == 0 ? b0 : b1;
      bi = daxpy_elem(bi, -u, sA[i + k * STOP], idx, len, lanes);
    }
  }
  if (lane < m) bc[lane] = b0;
  if (lane + 32 < m) bc[lane + 32] = b1;
}

// Left side, op(A) = A^T: trsm_ltl / trsm_ltu base cases (src/trsm.rs:176-188, 215-227).
constexpr int TCOLS = 32;  // right-hand sides per block in the transposed base case

template <bool LOWER>
__global__ void __launch_bounds__(TCOLS)
left_t_base(int m, int64_t n, bool unit, const double *__restrict__ A, int64_t lda, double *B,
            int64_t ldb, const int32_t *info) {
  __shared__ double sA[STOP * STOP];
  __shared__ double sB[STOP * TCOLS];
  if (stop_flag(info)) return;
  load_tri(sA, A, lda, m);
  const int64_t c0 = (int64_t)blockIdx.x * TCOLS;
  const int nc = (int)imin(TCOLS, n - c0);
  for (int e = threadIdx.x; e < m * TCOLS; e += blockDim.x) {
    const int i = e % m, c = e / m;
    sB[c + i * TCOLS] = c < nc ? B[i + (c0 + c) * ldb] : 0.0;
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c < nc) {
    for (int step = 0; step < m; ++step) {
      const int i = LOWER ? m - 1 - step : step;
      double t = sB[c + i * TCOLS];
      if (LOWER) {
        for (int k = i + 1; k < m; ++k) t = sub_prod(t, sA[k + i * STOP], sB[c + k * TCOLS]);
      } else {
        for (int k = 0; k < i; ++k) t = sub_prod(t, sA[k + i * STOP], sB[c + k * TCOLS]);
      }
      if (!unit) t = t / sA[i + i * STOP];
      sB[c + i * TCOLS] = t;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < m * TCOLS; e += blockDim.x) {
    const int i = e % m, cc = e / m;
    if (cc < nc) B[i + (c0 + cc) * ldb] = sB[cc + i * TCOLS];
  }
}

// Right side base cases (src/trsm.rs:253-273, 285-305, 317-337, 349-369).
// V: 0 = rnl, 1 = rnu, 2 = rtl, 3 = rtu.
template <int V>
__global__ void __launch_bounds__(128)
right_base(int64_t m, int n, bool unit, const double *__restrict__ A, int64_t lda, double *B,
           int64_t ldb, const int32_t *info) {
  __shared__ double sA[STOP * STOP];
  if (stop_flag(info)) return;
  load_tri(sA, A, lda, n);
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  constexpr bool descending = (V == 0 || V == 3);
  for (int step = 0; step < n; ++step) {
    const int j = descending ? n - 1 - step : step;
    double bj = B[i + j * ldb];
    const int k0 = descending ? j + 1 : 0;
    const int k1 = descending ? n : j;
    for (int k = k0; k < k1; ++k) {
      // rnl/rnu read a(k, j); rtl/rtu read a(j, k)
      const double akj = (V <= 1) ? sA[k + j * STOP] : sA[j + k * STOP];
      if (akj != 0.0) bj = sub_prod(bj, akj, B[i + k * ldb]);
    }
    if (!unit) bj = __dmul_rn(bj, 1.0 / sA[j + j * STOP]);
    B[i + j * ldb] = bj;
  }
}

struct Ctx {
  cudaStream_t s;
  bool unit;
  int lanes;
  const int32_t *info;
};

int base_left_n(const Ctx &c, bool lower, int64_t m, int64_t n, const double *A, int64_t lda, double *B,
                int64_t ldb) {
  ProfScope prof(c.s, "trsm_base", (double)m * m * n);
  const int warps = 8;
  const unsigned g = (unsigned)cdiv(n, warps);
  if (lower)
    left_n_base<true><<<g, 32 * warps, 0, c.s>>>((int)m, n, c.unit, A, lda, B, ldb, c.lanes, c.info);
  else
    left_n_base<false><<<g, 32 * warps, 0, c.s>>>((int)m, n, c.unit, A, lda, B, ldb, c.lanes, c.info);
  BOLA_CHECK_LAUNCH();
  return 0;
}

int base_left_t(const Ctx &c, bool lower, int64_t m, int64_t n, const double *A, int64_t lda, double *B,
                int64_t ldb) {
  ProfScope prof(c.s, "trsm_base", (double)m * m * n);
  const unsigned g = (unsigned)cdiv(n, TCOLS);
  if (lower)
    left_t_base<true><<<g, TCOLS, 0, c.s>>>((int)m, n, c.unit, A, lda, B, ldb, c.info);
  else
    left_t_base<false><<<g, TCOLS, 0, c.s>>>((int)m, n, c.unit, A, lda, B, ldb, c.info);
  BOLA_CHECK_LAUNCH();
  return 0;
}

int base_right(const Ctx &c, int v, int64_t m, int64_t n, const double *A, int64_t lda, double *B,
               int64_t ldb) {
  ProfScope prof(c.s, "trsm_base", (double)m * n * n);
  const unsigned g = (unsigned)cdiv(m, 128);
  switch (v) {
    case 0: right_base<0><<<g, 128, 0, c.s>>>(m, (int)n, c.unit, A, lda, B, ldb, c.info); break;
    case 1: right_base<1><<<g, 128, 0, c.s>>>(m, (int)n, c.unit, A, lda, B, ldb, c.info); break;
    case 2: right_base<2><<<g, 128, 0, c.s>>>(m, (int)n, c.unit, A, lda, B, ldb, c.info); break;
    default: right_base<3><<<g, 128, 0, c.s>>>(m, (int)n, c.unit, A, lda, B, ldb, c.info); break;
  }
  BOLA_CHECK_LAUNCH();
  return 0;
}

int gemm_upd(const Ctx &c, char ta, char tb, int64_t m, int64_t n, int64_t k, const double *A, int64_t lda,
             const double *B, int64_t ldb, double *C, int64_t ldc) {
  return dgemm_exact(c.s, ta, tb, m, n, k, -1.0, A, lda, B, ldb, 1.0, C, ldc, 64, c.info, 0);
}

// src/trsm.rs:95-131
int lnl(const Ctx &c, int64_t m, int64_t n, const double *a, int64_t lda, double *b, int64_t ldb) {
  if (m <= STOP) return base_left_n(c, true, m, n, a, lda, b, ldb);
  const int64_t m1 = m / 2, m2 = m - m1;
  BOLA_TRY(lnl(c, m1, n, a, lda, b, ldb));
  BOLA_TRY(gemm_upd(c, 'N', 'N', m2, n, m1, a + m1, lda, b, ldb, b + m1, ldb));
  return lnl(c, m2, n, a + m1 + m1 * lda, lda, b + m1, ldb);
}
// src/trsm.rs:135-170
int lnu(const Ctx &c, int64_t m, int64_t n, const double *a, int64_t lda, double *b, int64_t ldb) {
  if (m <= STOP) return base_left_n(c, false, m, n, a, lda, b, ldb);
  const int64_t m1 = m / 2, m2 = m - m1;
  BOLA_TRY(lnu(c, m2, n, a + m1 + m1 * lda, lda, b + m1, ldb));
  BOLA_TRY(gemm_upd(c, 'N', 'N', m1, n, m2, a + m1 * lda, lda, b + m1, ldb, b, ldb));
  return lnu(c, m1, n, a, lda, b, ldb);
}
// src/trsm.rs:174-209
int ltl(const Ctx &c, int64_t m, int64_t n, const double *a, int64_t lda, double *b, int64_t ldb) {
  if (m <= STOP) return base_left_t(c, true, m, n, a, lda, b, ldb);
  const int64_t m1 = m / 2, m2 = m - m1;
  BOLA_TRY(ltl(c, m2, n, a + m1 + m1 * lda, lda, b + m1, ldb));
  BOLA_TRY(gemm_upd(c, 'T', 'N', m1, n, m2, a + m1, lda, b + m1, ldb, b, ldb));
  return ltl(c, m1, n, a, lda, b, ldb);
}
// src/trsm.rs:213-248
int ltu(const Ctx &c, int64_t m, int64_t n, const double *a, int64_t lda, double *b, int64_t ldb) {
  if (m <= STOP) return base_left_t(c, false, m, n, a, lda, b, ldb);
  const int64_t m1 = m / 2, m2 = m - m1;
  BOLA_TRY(ltu(c, m1, n, a, lda, b, ldb));
  BOLA_TRY(gemm_upd(c, 'T', 'N', m2, n, m1, a + m1 * lda, lda, b, ldb, b + m1, ldb));
  return ltu(c, m2, n, a + m1 + m1 * lda, lda, b + m1, ldb);
}
// src/trsm.rs:252-280
int rnl(const Ctx &c, int64_t m, int64_t n, const double *a, int64_t lda, double *b, int64_t ldb) {
  if (n <= STOP) return base_right(c, 0, m, n, a, lda, b, ldb);
  const int64_t n1 = n / 2, n2 = n - n1;
  BOLA_TRY(rnl(c, m, n2, a + n1 + n1 * lda, lda, b + n1 * ldb, ldb));
  BOLA_TRY(gemm_upd(c, 'N', 'N', m, n1, n2, b + n1 * ldb, ldb, a + n1, lda, b, ldb));
  return rnl(c, m, n1, a, lda, b, ldb);
}
// src/trsm.rs:284-312
int rnu(const Ctx &c, int64_t m, int64_t n, const double *a, int64_t lda, double *b, int64_t ldb) {
  if (n <= STOP) return base_right(c, 1, m, n, a, lda, b, ldb);
  const int64_t n1 = n / 2, n2 = n - n1;
  BOLA_TRY(rnu(c, m, n1, a, lda, b, ldb));
  BOLA_TRY(gemm_upd(c, 'N', 'N', m, n2, n1, b, ldb, a + n1 * lda, lda, b + n1 * ldb, ldb));
  return rnu(c, m, n2, a + n1 + n1 * lda, lda, b + n1 * ldb, ldb);
}
// src/trsm.rs:316-344
int rtl(const Ctx &c, int64_t m, int64_t n, const double *a, int64_t lda, double *b, int64_t ldb) {
  if (n <= STOP) return base_right(c, 2, m, n, a, lda, b, ldb);
  const int64_t n1 = n / 2, n2 = n - n1;
  BOLA_TRY(rtl(c, m, n1, a, lda, b, ldb));
  BOLA_TRY(gemm_upd(c, 'N', 'T', m, n2, n1, b, ldb, a + n1, lda, b + n1 * ldb, ldb));
  return rtl(c, m, n2, a + n1 + n1 * lda, lda, b + n1 * ldb, ldb);
}
// src/trsm.rs:348-376
int rtu(const Ctx &c, int64_t m, int64_t n, const double *a, int64_t lda, double *b, int64_t ldb) {
  if (n <= STOP) return base_right(c, 3, m, n, a, lda, b, ldb);
  const int64_t n1 = n / 2, n2 = n - n1;
  BOLA_TRY(rtu(c, m, n2, a + n1 + n1 * lda, lda, b + n1 * ldb, ldb));
  BOLA_TRY(gemm_upd(c, 'N', 'T', m, n1, n2, b + n1 * ldb, ldb, a + n1 * lda, lda, b, ldb));
  return rtu(c, m, n1, a, lda, b, ldb);
}

}  // namespace

// src/trsm.rs:33-91: alpha pre-scale, then dispatch (case-insensitive).
int trsm_exact(cudaStream_t s, char side, char uplo, char transa, char diag, int64_t m, int64_t n,
               double alpha, const double *A, int64_t lda, double *B, int64_t ldb, const int32_t *info) {
  if (m <= 0 || n <= 0) return 0;
  if (alpha != 1.0) {
    ProfScope prof(s, "scale", (double)m * n);
    scale_matrix<<<(unsigned)cdiv(m * n, 256), 256, 0, s>>>(m, n, alpha, B, ldb, info);
    BOLA_CHECK_LAUNCH();
  }
  Ctx c{s, upc(diag) == 'U', lanes(), info};
  const bool left = upc(side) == 'L', upper = upc(uplo) == 'U', notrans = upc(transa) == 'N';
  if (left) {
    if (notrans) return upper ? lnu(c, m, n, A, lda, B, ldb) : lnl(c, m, n, A, lda, B, ldb);
    return upper ? ltu(c, m, n, A, lda, B, ldb) : ltl(c, m, n, A, lda, B, ldb);
  }
  if (notrans) return upper ? rnu(c, m, n, A, lda, B, ldb) : rnl(c, m, n, A, lda, B, ldb);
  return upper ? rtu(c, m, n, A, lda, B, ldb) : rtl(c, m, n, A, lda, B, ldb);
}

}  // namespace bola

extern "C" int bola_dtrsm(char side, char uplo, char transa, char diag, int64_t m, int64_t n,
                          double alpha, const double *a, int64_t lda, double *b, int64_t ldb,
                          bola_stream_t stream) {
  if (m < 0) return -5;
  if (n < 0) return -6;
  if (m == 0 || n == 0) return 0;
  const int64_t k = bola::upc(side) == 'L' ? m : n;
  if (lda < bola::imax(1, k)) return -9;
  if (ldb < bola::imax(1, m)) return -11;
  return bola::trsm_exact((cudaStream_t)stream, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb,
                          nullptr);
}
