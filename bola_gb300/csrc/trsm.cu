// trsm.cu — triangular solves with BOLA's recursion and rounding
// (src/trsm.rs:33-376).
//
// The host walks BOLA's recursion (halving down to 64) and issues the exact
// DGEMM for every off-diagonal block, so >97% of the flops run in the GEMM
// kernel.  The <=64 base cases run on the GPU with BOLA's per-element order:
//   left, no transpose  — column forward/back substitution with BOLA's daxpy
//                         (a warp per right-hand side, rows across lanes);
//   left, transpose     — dot-style substitution, one thread per column;
//   right               — column sweeps, one thread per row of B; the
//                         ascending ones (rnu, rtl) for n <= 32
//                         right-looking, a row over 4 lanes in registers.
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
    if (!nonzero64(bk)) continue;  // BOLA skips zero entries (src/trsm.rs:101,141)
    const double u = unit ? bk : bk / sA[k + k * STOP];
    if (k == lane) b0 = u;
    if (k == lane + 32) b1 = u;
    if (!nonzero64(u)) continue;  // daxpy returns early for a zero scale (src/utilities.rs:108)
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
// V: 0 = rnl, 1 = rnu, 2 = rtl, 3 = rtu.  A thread per row of B: the CTA's
// rows of B and the triangle are staged in shared memory (the row chains then
// never wait on global loads), and the reciprocals of the diagonal, which
// every row multiplies by, are formed once per CTA.
constexpr int RB_ROWS = 128;

inline size_t right_base_smem(int n) { return ((size_t)n * n + n + (size_t)RB_ROWS * n) * sizeof(double); }

template <int V>
__global__ void __launch_bounds__(RB_ROWS)
right_base(int64_t m, int n, bool unit, const double *__restrict__ A, int64_t lda, double *B,
           int64_t ldb, const int32_t *info) {
  extern __shared__ double rb_smem[];
  double *sA = rb_smem;      // n x n, ld n
  double *rd = sA + n * n;   // 1 / a(j, j)
  double *sB = rd + n;       // column k of the CTA's rows at sB[k * RB_ROWS]
  if (stop_flag(info)) return;
  const int64_t i0 = (int64_t)blockIdx.x * RB_ROWS;
  const int rows = (int)imin(RB_ROWS, m - i0);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) sA[e] = A[(e % n) + (int64_t)(e / n) * lda];
  for (int e = threadIdx.x; e < RB_ROWS * n; e += blockDim.x) {
    const int r = e % RB_ROWS, k = e / RB_ROWS;
    sB[e] = r < rows ? B[(i0 + r) + (int64_t)k * ldb] : 0.0;
  }
  __syncthreads();
  if (!unit && threadIdx.x < n) rd[threadIdx.x] = 1.0 / sA[threadIdx.x * (n + 1)];
  __syncthreads();
  constexpr bool descending = (V == 0 || V == 3);
  if (threadIdx.x < rows) {
    double *b = sB + threadIdx.x;
    for (int step = 0; step < n; ++step) {
      const int j = descending ? n - 1 - step : step;
      double bj = b[j * RB_ROWS];
      const int k0 = descending ? j + 1 : 0;
      const int k1 = descending ? n : j;
      for (int k = k0; k < k1; ++k) {
        // rnl/rnu read a(k, j); rtl/rtu read a(j, k)
        const double akj = (V <= 1) ? sA[k + j * n] : sA[j + k * n];
        if (nonzero64(akj)) bj = sub_prod(bj, akj, b[k * RB_ROWS]);
      }
      if (!unit) bj = __dmul_rn(bj, rd[j]);
      b[j * RB_ROWS] = bj;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < RB_ROWS * n; e += blockDim.x) {
    const int r = e % RB_ROWS, k = e / RB_ROWS;
    if (r < rows) B[(i0 + r) + (int64_t)k * ldb] = sB[e];
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

// The ascending right base cases (rnu, rtl) for n <= 32, right-looking: once
// b_k is final it is subtracted from every later column of the row, so each
// b_j still receives its updates in ascending k and then its scale, exactly as
// in BOLA's column sweep.  A row is spread over RL = 4 lanes, lane q holding
// columns q, q+4, ..., q+28 in registers: b_k is finished by its lane and
// broadcast by a shuffle, and each lane updates its own later columns.  The
// FP64 pipe retires a warp instruction in the same time whether 1 or 32 lanes
// work, and a row's work is one dependent sweep; spreading a row over 4 lanes
// cuts the instructions on a warp's path about 3.5-fold.
constexpr int RL = 4;             // lanes per row
constexpr int RA_THREADS = 64;    // 16 rows per CTA
constexpr int RA_ROWS = RA_THREADS / RL;

template <int V>
__global__ void __launch_bounds__(RA_THREADS)
right_base_asc32(int64_t m, int n, bool unit, const double *__restrict__ A, int64_t lda, double *B, int64_t ldb,
                 const int32_t *info) {
  static_assert(V == 1 || V == 2, "ascending variants only");
  __shared__ double sA[32 * 33];  // a(r, c) at sA[r + 33 c]
  __shared__ double rd[32];
  if (stop_flag(info)) return;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) sA[(e % n) + (e / n) * 33] = A[(e % n) + (int64_t)(e / n) * lda];
  __syncthreads();
  if (!unit && threadIdx.x < n) rd[threadIdx.x] = 1.0 / sA[threadIdx.x * 34];
  __syncthreads();
  const int lane = threadIdx.x & 31, q = lane & (RL - 1), base = lane & ~(RL - 1);
  const int64_t i = (int64_t)blockIdx.x * RA_ROWS + threadIdx.x / RL;
  const bool row = i < m;  // lanes of a missing row still take part in the shuffles
  double b[32 / RL];
#pragma unroll
  for (int c = 0; c < 32 / RL; ++c) {
    const int j = q + RL * c;
    b[c] = (row && j < n) ? B[i + (int64_t)j * ldb] : 0.0;
  }
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    if (k < n) {
      if (!unit && q == (k & (RL - 1))) b[k / RL] = __dmul_rn(b[k / RL], rd[k]);
      const double bk = __shfl_sync(0xffffffffu, b[k / RL], base + (k & (RL - 1)));
#pragma unroll
      for (int c = 0; c < 32 / RL; ++c) {
        const int j = q + RL * c;
        if (j > k && j < n) {
          const double a = (V == 1) ? sA[k + j * 33] : sA[j + k * 33];  // rnu: a(k, j); rtl: a(j, k)
          const double u = sub_prod(b[c], a, bk);
          b[c] = nonzero64(a) ? u : b[c];  // BOLA skips a zero a
        }
      }
    }
  }
  if (!row) return;
#pragma unroll
  for (int c = 0; c < 32 / RL; ++c) {
    const int j = q + RL * c;
    if (j < n) B[i + (int64_t)j * ldb] = b[c];
  }
}

template <int V>
int launch_right_base(const Ctx &c, int64_t m, int64_t n, const double *A, int64_t lda, double *B, int64_t ldb) {
  if constexpr (V == 1 || V == 2) {
    if (n <= 32) {
      right_base_asc32<V><<<(unsigned)cdiv(m, RA_ROWS), RA_THREADS, 0, c.s>>>(m, (int)n, c.unit, A, lda, B, ldb,
                                                                             c.info);
      BOLA_CHECK_LAUNCH();
      return 0;
    }
  }
  const size_t smem = right_base_smem((int)n);
  if (smem > 48 * 1024) BOLA_TRY_CUDA(cudaFuncSetAttribute(right_base<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  right_base<V><<<(unsigned)cdiv(m, RB_ROWS), RB_ROWS, smem, c.s>>>(m, (int)n, c.unit, A, lda, B, ldb, c.info);
  BOLA_CHECK_LAUNCH();
  return 0;
}

int base_right(const Ctx &c, int v, int64_t m, int64_t n, const double *A, int64_t lda, double *B,
               int64_t ldb) {
  ProfScope prof(c.s, "trsm_base", (double)m * n * n);
  switch (v) {
    case 0: return launch_right_base<0>(c, m, n, A, lda, B, ldb);
    case 1: return launch_right_base<1>(c, m, n, A, lda, B, ldb);
    case 2: return launch_right_base<2>(c, m, n, A, lda, B, ldb);
    default: return launch_right_base<3>(c, m, n, A, lda, B, ldb);
  }
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
