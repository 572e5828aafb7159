// potrf.cu — SYRK and Cholesky with BOLA's blocking and rounding
// (src/syrk.rs:17-249, src/potrf.rs:101-181, src/potrf2.rs:25-80).
//
// SYRK: BOLA walks 32x32 blocks of C and 32-deep blocks of K.  Off-diagonal
// blocks go through its gemm with K = 32, i.e. exactly the exact DGEMM with a
// 32-deep chunk, restricted to the strictly upper / lower block triangle.  The
// diagonal blocks use BOLA's syrk_kernel: per element a chain of daxpy
// updates ('N') or of 32-deep dot products ('T') — one thread per element.
//
// POTRF is BOLA's blocked Cholesky (NB = 32): diagonal SYRK, the 32x32
// potrf2 inside one CTA's shared memory, the panel GEMM and the triangular
// solve.  Below n = 320 the steps run in BOLA's left-looking order; from 320
// on the same per-element sums are formed right-looking with look-ahead on
// two streams (potrf_blocked below says why the results are identical).  The
// 'L' potrf2 block runs column by column with BOLA's fused/unfused pattern
// per element; 'U' and failing blocks use BOLA's recursion.
#include "common.cuh"

namespace bola {
namespace {

constexpr int NB = 32;  // src/syrk.rs:9, src/potrf.rs:8

__global__ void syrk_beta(bool upper, int64_t n, double beta, double *C, int64_t ldc, const int32_t *info) {
  if (stop_flag(info)) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int64_t i = e % n, j = e / n;
  if (upper ? i > j : i < j) return;
  double &c = C[i + j * ldc];
  c = beta == 0.0 ? 0.0 : __dmul_rn(c, beta);
}

// Diagonal 32x32 blocks: blockIdx.y = block, blockIdx.x = column jj in the
// block, threadIdx.x = row ii.  Each element's chain over k keeps BOLA's
// order exactly and is FP64-latency-bound, so the 32 columns of a block run
// on 32 SMs.  A arrives in 32-deep chunks staged in shared memory; the next
// chunk is prefetched into registers while the current one is consumed.
__global__ void __launch_bounds__(NB)
syrk_diag(bool upper, bool trans_t, int64_t n, int64_t k, double alpha, const double *__restrict__ A,
          int64_t lda, double *C, int64_t ldc, int lanes, const int32_t *info) {
  __shared__ double sA[NB][NB + 1];  // 'N': sA[l][r] = A(j0 + r, p0 + l); 'T': sA[r][l] = A(p0 + l, j0 + r)
  __shared__ double tl[NB];          // 'N': alpha * A(j0 + jj, p0 + l), the column's multipliers
  if (stop_flag(info)) return;
  const int64_t j0 = (int64_t)blockIdx.y * NB;
  const int jb = (int)imin(NB, n - j0);
  const int jj = blockIdx.x, ii = threadIdx.x;
  if (jj >= jb) return;  // uniform over the CTA
  const bool active = ii < jb && !(upper ? ii > jj : ii < jj);
  // BOLA's daxpy for column jj: the element is in the fused vector body or the unfused tail
  const int64_t len = upper ? jj + 1 : jb - jj;
  const int64_t idx = upper ? ii : ii - jj;
  const bool fz = idx < (len & ~(int64_t)(lanes - 1));
  double pre[NB];
  auto fetch = [&](int64_t p0) {
    const int pb = (int)imin(NB, k - p0);
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      if (trans_t)  // column q of the block, depth row ii
        pre[q] = (q < jb && ii < pb) ? A[(p0 + ii) + (j0 + q) * lda] : 0.0;
      else  // depth column q, block row ii
        pre[q] = (q < pb && ii < jb) ? A[(j0 + ii) + (p0 + q) * lda] : 0.0;
    }
  };
  double *cp = C + (j0 + ii) + (j0 + jj) * ldc;
  double c = active ? *cp : 0.0;
  if (k > 0) fetch(0);
  for (int64_t p0 = 0; p0 < k; p0 += NB) {
    const int pb = (int)imin(NB, k - p0);
    __syncthreads();  // the previous chunk is consumed
#pragma unroll
    for (int q = 0; q < NB; ++q) sA[q][ii] = pre[q];  // both layouts: q is l ('N') or r ('T')
    __syncthreads();
    // one multiplier per lane, and which are non-zero (BOLA's daxpy skips a
    // zero scale): the chain below then issues one FP64 instruction per step,
    // the only one GB300's narrow FP64 pipe must serialise
    uint32_t nz = 0;
    if (!trans_t) {
      const double tv = ii < pb ? __dmul_rn(alpha, sA[ii][jj]) : 0.0;
      tl[ii] = tv;
      nz = __ballot_sync(0xffffffffu, nonzero64(tv));
    }
    __syncthreads();
    if (p0 + NB < k) fetch(p0 + NB);
    if (!active) continue;
    if (!trans_t) {
      // syrk_kernel 'N' (src/syrk.rs:201-222): C(:,jj) += (alpha*A(jj,l)) * A(:,l), BOLA's daxpy
      if (fz) {
#pragma unroll 4
        for (int l = 0; l < pb; ++l)
          if ((nz >> l) & 1u) c = fused(tl[l], sA[l][ii], c);
      } else {
        for (int l = 0; l < pb; ++l)
          if ((nz >> l) & 1u) c = add_prod(c, tl[l], sA[l][ii]);
      }
    } else {
      // syrk_kernel 'T' (src/syrk.rs:223-247): C(ii,jj) += alpha * dot(A(:,ii), A(:,jj))
      const double t = dot_exact(pb, &sA[ii][0], 1, &sA[jj][0], 1, lanes);
      c = add_prod(c, alpha, t);
    }
  }
  if (active) *cp = c;
}

// ---- potrf2 on one <=32 x 32 block in shared memory (src/potrf2.rs:36-80) ----
constexpr int LDS = NB;

// BOLA's recursion (halve, factor the leading half, trsm + syrk, factor the
// trailing half) walked with an explicit stack: device recursion would need
// more per-thread stack than the default.  Every thread runs the same walk.
// Returns 0 or the 1-based failing column inside the block.
//
// 'L': the reciprocal of each diagonal element, which the trsm of every
// enclosing level multiplies by, is formed once, by the thread that takes
// the square root, into rdg (indexed by the element's position in the block).
__device__ int p2_walk(bool upper, double *a0, double *rdg, int n, int lanes) {
  struct Frame {
    int off, n, phase;
  };
  Frame st[8];
  int sp = 0;
  st[0] = {0, n, 0};
  const int tid = threadIdx.x;
  while (sp >= 0) {
    Frame &f = st[sp];
    double *a = a0 + f.off + f.off * LDS;
    if (f.n == 0) {
      --sp;
      continue;
    }
    if (f.n == 1) {  // src/potrf2.rs:41-48
      const double a11 = a[0];
      __syncthreads();
      if (!(a11 > 0.0)) return f.off + 1;
      if (tid == 0) {
        const double d = sqrt(a11);
        a[0] = d;
        if (!upper) rdg[f.off] = 1.0 / d;
      }
      __syncthreads();
      --sp;
      continue;
    }
    const int n1 = f.n / 2, n2 = f.n - n1;
    if (f.phase == 0) {
      f.phase = 1;
      st[++sp] = {f.off, n1, 0};
      continue;
    }
    if (f.phase == 2) {
      --sp;
      continue;
    }
    double *a22 = a + n1 + n1 * LDS;
    if (upper) {
      double *a12 = a + n1 * LDS;
      // trsm('L','U','T','N', n1, n2, 1, a11, a12): trsm_ltu base, a thread per column
      if (tid < n2) {
        for (int i = 0; i < n1; ++i) {
          double t = a12[i + tid * LDS];
          for (int k = 0; k < i; ++k) t = sub_prod(t, a[k + i * LDS], a12[k + tid * LDS]);
          t = t / a[i + i * LDS];
          a12[i + tid * LDS] = t;
        }
      }
      __syncthreads();
      // syrk('U','T', n2, n1, -1, a12, 1, a22): dot path
      for (int e = tid; e < n2 * n2; e += blockDim.x) {
        const int ii = e % n2, jj = e / n2;
        if (ii > jj) continue;
        const double t = dot_exact(n1, a12 + ii * LDS, 1, a12 + jj * LDS, 1, lanes);
        a22[ii + jj * LDS] = add_prod(a22[ii + jj * LDS], -1.0, t);
      }
    } else {
      double *a21 = a + n1;
      // trsm('R','L','T','N', n2, n1, 1, a11, a21): trsm_rtl base, a thread per row
      if (tid < n2) {
        for (int j = 0; j < n1; ++j) {
          double b = a21[tid + j * LDS];
          for (int k = 0; k < j; ++k) {
            const double ajk = a[j + k * LDS];
            if (nonzero64(ajk)) b = sub_prod(b, ajk, a21[tid + k * LDS]);
          }
          b = __dmul_rn(b, rdg[f.off + j]);
          a21[tid + j * LDS] = b;
        }
      }
      __syncthreads();
      // syrk('L','N', n2, n1, -1, a21, 1, a22): daxpy path
      for (int e = tid; e < n2 * n2; e += blockDim.x) {
        const int ii = e % n2, jj = e / n2;
        if (ii < jj) continue;
        double c = a22[ii + jj * LDS];
        for (int l = 0; l < n1; ++l) {
          const double t = -a21[jj + l * LDS];
          if (nonzero64(t)) c = daxpy_elem(c, t, a21[ii + l * LDS], ii - jj, n2 - jj, lanes);
        }
        a22[ii + jj * LDS] = c;
      }
    }
    __syncthreads();
    f.phase = 2;
    st[++sp] = {f.off + n1, n2, 0};
  }
  return 0;
}

// 128 threads: one warp per SMSP, so the SYRK steps' FP64 work never queues
// two warps on one sub-partition's FP64 pipe.
constexpr int P2T = 128;
constexpr int P2E = (LDS * (LDS + 1) / 2 + P2T - 1) / P2T;  // lower-triangle elements per thread

// Which updates of element (i, j) (i >= j) BOLA's recursion makes fused: bit l
// set if the update from column l < j is the fused body of a daxpy.  In
// p2_walk every update of (i, j) comes from a column l < j, in increasing l:
// first from the SYRK of each frame whose leading half holds l and whose
// trailing half holds i and j (a daxpy over that half's column jj: element
// idx = ii - jj of len = n2 - jj, fused below len rounded down to the SIMD
// width), then, in the frame that separates i from j, from its TRSM (unfused
// b - a*x for l in [frame start, j)), after which (i, j) is scaled by 1/l_jj.
__device__ uint32_t fused_updates(int i, int j, int n, int lanes) {
  uint32_t m = 0;
  int off = 0, nn = n;
  while (nn > 1) {
    const int n1 = nn / 2, n2 = nn - n1, split = off + n1;
    if (j >= split) {  // (i, j) in the trailing half: SYRK from l in [off, split)
      const int jj = j - split, idx = i - j, len = n2 - jj;
      if (idx < (len & ~(lanes - 1))) m |= ((1u << n1) - 1u) << off;
      off = split;
      nn = n2;
    } else if (i >= split) {  // below the leading half: the TRSM, unfused
      break;
    } else {
      nn = n1;
    }
  }
  return m;
}

// potrf2 'L' of the block in shared memory, right-looking: column l is
// finished (square root, 1/l_ll, the column scaled), then every element
// (i, j > l) takes its update from column l, fused or not as BOLA's recursion
// does it.  Every element sees BOLA's operations in BOLA's order, so the factor
// is bit-identical; the dependent chain per column is one square root and
// one reciprocal instead of the recursion's chains of solves.  Returns 0 or
// the 1-based failing column; the block is then not in BOLA's state (the
// caller redoes it with p2_walk).
__device__ int p2_right_looking(double *a, double *rdg, int n, int lanes) {
  __shared__ int fail;
  const int tid = threadIdx.x;
  int ei[P2E], ej[P2E];
  uint32_t em[P2E];
#pragma unroll
  for (int s = 0; s < P2E; ++s) {  // element e = tid + s * P2T of the packed lower triangle, column by column
    int e = tid + s * P2T, j = 0;
    while (j < n && e >= n - j) {
      e -= n - j;
      ++j;
    }
    ei[s] = j < n ? j + e : -1;
    ej[s] = j;
    em[s] = j < n ? fused_updates(j + e, j, n, lanes) : 0u;
  }
  if (tid == 0) fail = 0;
  __syncthreads();
  for (int l = 0; l < n; ++l) {
    if (tid == 0) {
      const double d = a[l + l * LDS];
      const long long db = __double_as_longlong(d);
      if (db > 0 && db <= 0x7ff0000000000000ll) {  // d > 0, not NaN
        const double r = sqrt(d);
        a[l + l * LDS] = r;
        rdg[l] = 1.0 / r;
      } else {
        fail = l + 1;
      }
    }
    __syncthreads();
    if (fail) return fail;
    const double rl = rdg[l];
#pragma unroll
    for (int s = 0; s < P2E; ++s)
      if (ej[s] == l && ei[s] > l) a[ei[s] + l * LDS] = __dmul_rn(a[ei[s] + l * LDS], rl);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < P2E; ++s) {
      const int i = ei[s], j = ej[s];
      if (i < 0 || j <= l) continue;
      const double ljl = a[j + l * LDS];
      if (!nonzero64(ljl)) continue;  // BOLA skips a zero multiplier
      const double lil = a[i + l * LDS];
      double &c = a[i + j * LDS];
      c = fused_or_unfused((em[s] >> l) & 1u, -ljl, lil, c);  // unfused: c + (-l_jl) l_il = c - l_jl l_il
    }
    __syncthreads();
  }
  return 0;
}

__global__ void __launch_bounds__(P2T)
potrf2_block(bool upper, int n, double *A, int64_t lda, int32_t *info, int32_t col0, int lanes) {
  __shared__ double a[LDS * LDS];
  __shared__ double a0[LDS * LDS];  // the input, for a failing 'L' block
  __shared__ double rdg[LDS];
  if (stop_flag(info)) return;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const double v = A[(e % n) + (e / n) * lda];
    a[(e % n) + (e / n) * LDS] = v;
    a0[(e % n) + (e / n) * LDS] = v;
  }
  __syncthreads();
  int r = upper ? p2_walk(true, a, rdg, n, lanes) : p2_right_looking(a, rdg, n, lanes);
  if (!upper && r) {  // BOLA's state at a failure is its recursion's: redo the block that way
    __syncthreads();
    for (int e = threadIdx.x; e < LDS * LDS; e += blockDim.x) a[e] = a0[e];
    __syncthreads();
    r = p2_walk(false, a, rdg, n, lanes);
  }
  __syncthreads();
  // BOLA stops at the failing column with everything before it written back.
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[(e % n) + (e / n) * lda] = a[(e % n) + (e / n) * LDS];
  if (r && threadIdx.x == 0) *info = col0 + r;
}

__global__ void zero_i32(int32_t *p) { *p = 0; }

}  // namespace

int syrk_exact(cudaStream_t s, char uplo, char trans, int64_t n, int64_t k, double alpha, const double *A,
               int64_t lda, double beta, double *C, int64_t ldc, const int32_t *info) {
  const bool upper = upc(uplo) == 'U', tt = upc(trans) != 'N';
  if (n <= 0 || ((alpha == 0.0 || k <= 0) && beta == 1.0)) return 0;
  if (beta != 1.0) {
    ProfScope prof(s, "syrk_beta", (double)n * n);
    syrk_beta<<<(unsigned)cdiv(n * n, 256), 256, 0, s>>>(upper, n, beta, C, ldc, info);
    BOLA_CHECK_LAUNCH();
  }
  if (alpha == 0.0 || k <= 0) return 0;
  if (n > NB) {
    BOLA_TRY(dgemm_exact(s, tt ? 'T' : 'N', tt ? 'N' : 'T', n, n, k, alpha, A, lda, A, lda, 1.0, C, ldc, NB,
                         info, upper ? 1 : 2));
  }
  ProfScope prof(s, "syrk_diag", (double)imin(n, NB) * (imin(n, NB) + 1) * (double)k * (double)cdiv(n, NB));
  syrk_diag<<<dim3(NB, (unsigned)cdiv(n, NB)), NB, 0, s>>>(upper, tt, n, k, alpha, A, lda, C, ldc, lanes(), info);
  BOLA_CHECK_LAUNCH();
  return 0;
}

int potrf2_rec(cudaStream_t s, char uplo, int64_t n, double *A, int64_t lda, int32_t *info, int32_t col0) {
  const bool upper = upc(uplo) == 'U';
  if (n == 0) return 0;
  if (n <= NB) {
    ProfScope prof(s, "potrf2_block", (double)n * n * n / 3.0);
    potrf2_block<<<1, P2T, 0, s>>>(upper, (int)n, A, lda, info, col0, lanes());
    BOLA_CHECK_LAUNCH();
    return 0;
  }
  const int64_t n1 = n / 2, n2 = n - n1;
  BOLA_TRY(potrf2_rec(s, uplo, n1, A, lda, info, col0));
  double *a22 = A + n1 + n1 * lda;
  if (upper) {
    BOLA_TRY(trsm_exact(s, 'L', 'U', 'T', 'N', n1, n2, 1.0, A, lda, A + n1 * lda, lda, info));
    BOLA_TRY(syrk_exact(s, 'U', 'T', n2, n1, -1.0, A + n1 * lda, lda, 1.0, a22, lda, info));
  } else {
    BOLA_TRY(trsm_exact(s, 'R', 'L', 'T', 'N', n2, n1, 1.0, A, lda, A + n1, lda, info));
    BOLA_TRY(syrk_exact(s, 'L', 'N', n2, n1, -1.0, A + n1, lda, 1.0, a22, lda, info));
  }
  return potrf2_rec(s, uplo, n2, a22, lda, info, col0 + (int32_t)n1);
}

namespace {

// One launch of the diagonal-block chain advance: the diagonal blocks of the
// nt x nt trailing matrix at C advance over the 32 columns (rows for 'U') at
// src.
int advance_diag(cudaStream_t s, bool upper, int64_t nt, const double *src, int64_t lda, double *C, int lan,
                 const int32_t *info) {
  if (nt <= 0) return 0;
  ProfScope prof(s, "syrk_diag", (double)NB * (NB + 1) * (double)NB * (double)cdiv(nt, NB));
  syrk_diag<<<dim3(NB, (unsigned)cdiv(nt, NB)), NB, 0, s>>>(upper, upper, nt, NB, -1.0, src, lda, C, lda, lan, info);
  BOLA_CHECK_LAUNCH();
  return 0;
}

// The 64-deep chunk starting at column (row, for 'U') c0 applied to the block
// column (row) at t and the rows below it (columns right of it): one block
// column wide.
int chunk_narrow(cudaStream_t s, bool upper, int64_t n, int64_t c0, int64_t t, double *A, int64_t lda,
                 const int32_t *info) {
  const int64_t below = n - t - NB;
  if (below <= 0) return 0;
  if (upper)
    return dgemm_exact(s, 'T', 'N', NB, below, 2 * NB, -1.0, A + c0 + t * lda, lda, A + c0 + (t + NB) * lda, lda, 1.0,
                       A + t + (t + NB) * lda, lda, 64, info, 0);
  return dgemm_exact(s, 'N', 'T', below, NB, 2 * NB, -1.0, A + (t + NB) + c0 * lda, lda, A + t + c0 * lda, lda, 1.0,
                     A + (t + NB) + t * lda, lda, 64, info, 0);
}

// The same chunk on every block column (row) from t on: block-triangular.
int chunk_wide(cudaStream_t s, bool upper, int64_t n, int64_t c0, int64_t t, double *A, int64_t lda,
               const int32_t *info) {
  const int64_t nt = n - t;
  if (nt <= NB) return 0;
  if (upper)
    return dgemm_exact(s, 'T', 'N', nt, nt, 2 * NB, -1.0, A + c0 + t * lda, lda, A + c0 + t * lda, lda, 1.0,
                       A + t + t * lda, lda, 64, info, 1);
  return dgemm_exact(s, 'N', 'T', nt, nt, 2 * NB, -1.0, A + t + c0 * lda, lda, A + t + c0 * lda, lda, 1.0,
                     A + t + t * lda, lda, 64, info, 2);
}

// Block p's own work: potrf2 of its diagonal block, the half chunk [j-32, j)
// of its GEMM when p is odd, and its triangular solve.
int block_step(cudaStream_t s, bool upper, int64_t n, int64_t j, double *A, int64_t lda, int32_t *info) {
  const int64_t jb = imin(NB, n - j), t = j + jb, n_rem = n - t;
  double *ajj = A + j + j * lda;
  BOLA_TRY(potrf2_rec(s, upper ? 'U' : 'L', jb, ajj, lda, info, (int32_t)j));
  if (n_rem == 0) return 0;
  const bool odd = (j / NB) & 1;
  if (upper) {
    if (odd)
      BOLA_TRY(dgemm_exact(s, 'T', 'N', jb, n_rem, NB, -1.0, A + (j - NB) + j * lda, lda, A + (j - NB) + t * lda, lda,
                           1.0, A + j + t * lda, lda, 64, info, 0));
    return trsm_exact(s, 'L', 'U', 'T', 'N', jb, n_rem, 1.0, ajj, lda, A + j + t * lda, lda, info);
  }
  if (odd)
    BOLA_TRY(dgemm_exact(s, 'N', 'T', n_rem, jb, NB, -1.0, A + t + (j - NB) * lda, lda, A + j + (j - NB) * lda, lda,
                         1.0, A + t + j * lda, lda, 64, info, 0));
  return trsm_exact(s, 'R', 'L', 'T', 'N', n_rem, jb, 1.0, ajj, lda, A + t + j * lda, lda, info);
}

}  // namespace

// BOLA's left-looking Cholesky (src/potrf.rs:114-178) computes block column p
// from all earlier columns at step p: a SYRK chain of length 32p for the
// diagonal block and a GEMM with K = 32p for the rows below it, both one
// after the other on the critical path.  Here the same sums are formed
// right-looking, as soon as their inputs are final:
//  - every element's SYRK chain runs in column order, so after block p is
//    final all later diagonal blocks advance their chains by its 32 columns;
//  - BOLA's GEMM forms one 64-deep chunk at a time (c = fma(alpha, acc, c),
//    chunks from k = 0), so when a chunk's 64 columns are final it is applied
//    to every later block column in one block-triangular GEMM; a block whose
//    K ends in a half chunk gets that 32-deep chunk at its own step.  The
//    8x4 edge classification depends only on n (block origins are multiples
//    of 32), so edge elements stay edge elements.
// The arithmetic per element is BOLA's, in BOLA's order: results are
// bit-identical.  What differs is the state after a failure: BOLA leaves the
// columns after the failing block untouched, so the lower (upper) part from
// the failing block's first sub-diagonal row (column) on is restored from a
// copy of A taken at entry.
//
// Look-ahead: the critical path (potrf2, half chunk, trsm of block p, then
// the chain advance and chunk for block p+1 only) runs on a high-priority
// stream; the advance of blocks >= p+2 and the chunk GEMM on block columns
// >= p+2 run on a low-priority stream behind it.  Ordering: block p+1's
// advance waits for the previous wide advance (the chains stay in column
// order), and block p's half chunk / trsm wait for the last wide chunk that
// covered block column p.
__global__ void potrf_restore(bool upper, int64_t n, const double *__restrict__ bk, double *A, int64_t lda,
                              const int32_t *info) {
  const int32_t f = *info;
  if (f == 0) return;
  const int64_t jf = (int64_t)((f - 1) / NB) * NB;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n, c = e / n;
    const int64_t r = upper ? c : i, q = upper ? i : c;  // r: position along the factor's rows, q: its columns
    if (q >= jf && r >= q && r >= jf + NB) A[i + c * lda] = bk[e];
  }
}

// BOLA's blocking literally (left-looking), for small orders: below ~320 the
// look-ahead streams, the input copy and the extra launches of the
// right-looking form cost more than its shorter critical path saves.
int potrf_left_looking(cudaStream_t s, bool upper, int64_t n, double *A, int64_t lda, int32_t *info) {
  for (int64_t j = 0; j < n; j += NB) {
    const int64_t jb = imin(NB, n - j), n_rem = n - j - jb;
    double *ajj = A + j + j * lda;
    if (upper) {
      BOLA_TRY(syrk_exact(s, 'U', 'T', jb, j, -1.0, A + j * lda, lda, 1.0, ajj, lda, info));
      BOLA_TRY(potrf2_rec(s, 'U', jb, ajj, lda, info, (int32_t)j));
      if (n_rem > 0) {
        BOLA_TRY(dgemm_exact(s, 'T', 'N', jb, n_rem, j, -1.0, A + j * lda, lda, A + (j + jb) * lda, lda, 1.0,
                             A + j + (j + jb) * lda, lda, 64, info, 0));
        BOLA_TRY(trsm_exact(s, 'L', 'U', 'T', 'N', jb, n_rem, 1.0, ajj, lda, A + j + (j + jb) * lda, lda, info));
      }
    } else {
      BOLA_TRY(syrk_exact(s, 'L', 'N', jb, j, -1.0, A + j, lda, 1.0, ajj, lda, info));
      BOLA_TRY(potrf2_rec(s, 'L', jb, ajj, lda, info, (int32_t)j));
      if (n_rem > 0) {
        BOLA_TRY(dgemm_exact(s, 'N', 'T', n_rem, jb, j, -1.0, A + j + jb, lda, A + j, lda, 1.0,
                             A + j + jb + j * lda, lda, 64, info, 0));
        BOLA_TRY(trsm_exact(s, 'R', 'L', 'T', 'N', n_rem, jb, 1.0, ajj, lda, A + j + jb + j * lda, lda, info));
      }
    }
  }
  return 0;
}

constexpr int64_t RIGHT_LOOKING_MIN_N = 320;

int potrf_blocked(cudaStream_t s, char uplo, int64_t n, double *A, int64_t lda, int32_t *info) {
  const bool upper = uplo == 'U';
  if (n < RIGHT_LOOKING_MIN_N) {
    {
      ProfScope prof(s, "info_init");
      zero_i32<<<1, 1, 0, s>>>(info);
    }
    BOLA_CHECK_LAUNCH();
    if (NB >= n) return potrf2_rec(s, uplo, n, A, lda, info, 0);
    return potrf_left_looking(s, upper, n, A, lda, info);
  }
  const int lan = lanes();
  Scratch bk;
  BOLA_TRY(bk.alloc((size_t)n * n * sizeof(double), s));
  LookAhead *la = la_acquire();
  cudaStream_t sp = la ? la->sp : s, su = la ? la->su : s;
  auto on = [&](cudaEvent_t e, cudaStream_t from, cudaStream_t to) -> int {
    if (!la || from == to) return 0;
    BOLA_TRY_CUDA(cudaEventRecord(e, from));
    BOLA_TRY_CUDA(cudaStreamWaitEvent(to, e, 0));
    return 0;
  };
  auto run = [&]() -> int {
    if (la) {
      BOLA_TRY_CUDA(cudaEventRecord(la->ev[0], s));
      BOLA_TRY_CUDA(cudaStreamWaitEvent(sp, la->ev[0], 0));
      BOLA_TRY_CUDA(cudaStreamWaitEvent(su, la->ev[0], 0));
    }
    {
      ProfScope prof(sp, "info_init");
      zero_i32<<<1, 1, 0, sp>>>(info);
    }
    BOLA_CHECK_LAUNCH();
    BOLA_TRY_CUDA(cudaMemcpy2DAsync(bk.as<double>(), (size_t)n * sizeof(double), A, (size_t)lda * sizeof(double),
                                    (size_t)n * sizeof(double), (size_t)n, cudaMemcpyDeviceToDevice, sp));
    // events: ev[1] critical part of step q done; ev[2 + (q & 1)] wide advance of
    // step q done; ev[4 + ((q >> 1) & 1)] wide chunk of odd step q done
    bool syrk_pending = false;
    int64_t last_wide = -1;  // the last odd step whose wide chunk was issued
    for (int64_t j = 0, q = 0; j < n; j += NB, ++q) {
      const int64_t t = j + NB, n_rem = n - t;
      // block column q last got a wide chunk from odd step q-2 (q odd) or q-3 (q even)
      const int64_t need = (q & 1) ? q - 2 : q - 3;
      if (la && need >= 1 && need <= last_wide)
        BOLA_TRY_CUDA(cudaStreamWaitEvent(sp, la->ev[4 + ((need >> 1) & 1)], 0));
      BOLA_TRY(block_step(sp, upper, n, j, A, lda, info));
      if (n_rem <= 0) break;
      if (la && syrk_pending) BOLA_TRY_CUDA(cudaStreamWaitEvent(sp, la->ev[2 + ((q - 1) & 1)], 0));
      const double *src_n = upper ? A + j + t * lda : A + t + j * lda;
      BOLA_TRY(advance_diag(sp, upper, imin(NB, n_rem), src_n, lda, A + t + t * lda, lan, info));
      const bool odd = q & 1;
      if (odd) BOLA_TRY(chunk_narrow(sp, upper, n, j - NB, t, A, lda, info));
      syrk_pending = false;
      if (n_rem > NB) {
        BOLA_TRY(on(la ? la->ev[1] : nullptr, sp, su));
        const int64_t t2 = t + NB;
        const double *src_w = upper ? A + j + t2 * lda : A + t2 + j * lda;
        BOLA_TRY(advance_diag(su, upper, n_rem - NB, src_w, lda, A + t2 + t2 * lda, lan, info));
        if (la) BOLA_TRY_CUDA(cudaEventRecord(la->ev[2 + (q & 1)], su));
        syrk_pending = true;
        if (odd) {
          BOLA_TRY(chunk_wide(su, upper, n, j - NB, t2, A, lda, info));
          if (la) BOLA_TRY_CUDA(cudaEventRecord(la->ev[4 + ((q >> 1) & 1)], su));
          last_wide = q;
        }
      }
    }
    BOLA_TRY(on(la ? la->ev[6] : nullptr, su, sp));
    {
      ProfScope prof(sp, "potrf_restore");
      potrf_restore<<<2 * (unsigned)num_sms(), 256, 0, sp>>>(upper, n, bk.as<double>(), A, lda, info);
    }
    BOLA_CHECK_LAUNCH();
    BOLA_TRY(on(la ? la->ev[7] : nullptr, sp, s));
    return 0;
  };
  const int st = run();
  if (la) {
    if (st != 0) {  // leave nothing of this call running on the look-ahead streams
      cudaStreamSynchronize(la->sp);
      cudaStreamSynchronize(la->su);
    }
    la_release(la);
  }
  return st;
}

}  // namespace bola

using namespace bola;

extern "C" {

int bola_dsyrk(char uplo, char trans, int64_t n, int64_t k, double alpha, const double *a, int64_t lda,
               double beta, double *c, int64_t ldc, bola_stream_t stream) {
  if (n < 0) return -3;
  if (k < 0) return -4;
  if (n == 0) return 0;
  const bool tt = upc(trans) != 'N';
  if (k > 0 && alpha != 0.0 && lda < imax(1, tt ? k : n)) return -7;
  if (ldc < imax(1, n)) return -10;
  return syrk_exact((cudaStream_t)stream, uplo, trans, n, k, alpha, a, lda, beta, c, ldc, nullptr);
}

int bola_dpotrf(char uplo, int64_t n, double *a, int64_t lda, int32_t *info, bola_stream_t stream) {
  if (uplo != 'U' && uplo != 'L') return -1;  // "Argument 1 to potrf had an illegal value" (src/potrf.rs:105-107)
  if (n < 0) return -2;
  if (lda < imax(n, 1)) return -4;  // "Argument 4 to potrf had an illegal value" (src/potrf.rs:108-110)
  return potrf_blocked((cudaStream_t)stream, uplo, n, a, lda, info);
}

int bola_dpotrf2(char uplo, int64_t n, double *a, int64_t lda, int32_t *info, bola_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (n < 0) return -2;
  if (lda < imax(n, 1)) return -4;
  {
    ProfScope prof(s, "info_init");
    zero_i32<<<1, 1, 0, s>>>(info);
  }
  BOLA_CHECK_LAUNCH();
  return potrf2_rec(s, uplo, n, a, lda, info, 0);
}

int bola_dpotrs(char uplo, int64_t n, int64_t nrhs, const double *fac, int64_t lda, double *b, int64_t ldb,
                bola_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (upc(uplo) != 'U' && upc(uplo) != 'L') return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < imax(1, n)) return -5;
  if (ldb < imax(1, n)) return -7;
  if (n == 0 || nrhs == 0) return 0;
  if (upc(uplo) == 'L') {
    BOLA_TRY(trsm_exact(s, 'L', 'L', 'N', 'N', n, nrhs, 1.0, fac, lda, b, ldb, nullptr));
    return trsm_exact(s, 'L', 'L', 'T', 'N', n, nrhs, 1.0, fac, lda, b, ldb, nullptr);
  }
  BOLA_TRY(trsm_exact(s, 'L', 'U', 'T', 'N', n, nrhs, 1.0, fac, lda, b, ldb, nullptr));
  return trsm_exact(s, 'L', 'U', 'N', 'N', n, nrhs, 1.0, fac, lda, b, ldb, nullptr);
}

}  // extern "C"
