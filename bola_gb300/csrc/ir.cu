// ir.cu — mixed-precision solve: low-precision LU on the tensor cores,
// FP64 iterative refinement (no BOLA counterpart; the FP64 answer it must
// reach is BOLA's getrf + trsm solve).
//
//   W = fl32(A S)                 S: power-of-two scale per 64-column block
//   P W = L U                     slu.cu (tcgen05 trailing updates)
//   x0 = S U^-1 L^-1 P b          FP32 triangular solves
//   repeat: r = b - A x           FP64 (the exact DGEMM)
//           berr = max_rhs ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf)
//           stop when berr <= tol; on a sweep gaining less than ~3x switch
//           to GMRES-IR, and when that stalls too, to the plain FP64 path
//           d = S U^-1 L^-1 P (r / ||r||) * ||r||;  x += d    (FP64 update)
// The residual, the update and the backward-error test are the only FP64
// steps.  Each FP32 triangular solve is one launch: a dataflow over 64-row
// blocks in which a CTA per block folds in the blocks solved before it as
// their flags appear, then applies the precomputed inverse of its diagonal
// block.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "mixed.cuh"
#include "sm100.cuh"

namespace cg = cooperative_groups;

namespace bola {
namespace {

constexpr int TB = 64;      // triangular-solve block (= LU block)
constexpr int MAXRHS = 32;  // right-hand sides per refinement sweep

// ---- scaling and conversion -------------------------------------------------------
// Per 64-column block the largest |a| (a CTA per block and slice of rows,
// every thread's loads of 4 columns in flight together), folded with 64-bit
// atomics into mbits as the bits of a non-negative double (they order like
// the values; mbits starts at zero); colblock_finish then turns it in place
// into the block's scale 2^-e with max|a| in [2^(e-1), 2^e).  A NaN is
// passed over, as fmax does.
__global__ void __launch_bounds__(256)
colblock_max(int64_t n, const double *__restrict__ A, int64_t lda, unsigned long long *mbits) {
  __shared__ double red[8];
  const int64_t c0 = (int64_t)blockIdx.x * TB, c1 = imin(n, c0 + TB);
  const int64_t rs = cdiv(n, (int64_t)gridDim.y), r0 = (int64_t)blockIdx.y * rs, r1 = imin(n, r0 + rs);
  double m = 0.0;
  for (int64_t c = c0; c < c1; c += 4)
    for (int64_t i = r0 + threadIdx.x; i < r1; i += 256) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = c + u < c1 ? fabs(A[i + (c + u) * lda]) : 0.0;
#pragma unroll
      for (int u = 0; u < 4; ++u) m = fmax(m, v[u]);
    }
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) m = fmax(m, red[w]);
    atomicMax(mbits + blockIdx.x, (unsigned long long)__double_as_longlong(m));
  }
}
__global__ void colblock_finish(int64_t nb, double *scale) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const double mm = scale[b];  // (the bits colblock_max left)
  int e = 0;
  frexp(mm, &e);
  scale[b] = (mm > 0.0 && isfinite(mm)) ? ldexp(1.0, -e) : 1.0;
}

// W = A S rounded to T (exact for T = double: S is a power of two per block).
template <typename T>
__global__ void convert_scaled(int64_t n, const double *__restrict__ A, int64_t lda, const double *scale,
                               T *__restrict__ W, int64_t ldw) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int64_t i = e % n, j = e / n;
  W[i + j * ldw] = (T)(A[i + j * lda] * scale[j / TB]);
}

// max|u_ii| and min|u_ii| of the low-precision U (one CTA): a cheap lower
// bound on the conditioning the refinement will face.
template <typename T>
__global__ void diag_extent(int64_t n, const T *__restrict__ W, int64_t ldw, double *out) {
  __shared__ double mx[32], mn[32];
  double a = 0.0, b = INFINITY;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = fabs((double)W[i + i * ldw]);
    a = fmax(a, v);
    b = fmin(b, v);
  }
  for (int off = 16; off > 0; off >>= 1) {
    a = fmax(a, __shfl_xor_sync(0xffffffffu, a, off));
    b = fmin(b, __shfl_xor_sync(0xffffffffu, b, off));
  }
  if ((threadIdx.x & 31) == 0) {
    mx[threadIdx.x >> 5] = a;
    mn[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      a = fmax(a, mx[w]);
      b = fmin(b, mn[w]);
    }
    out[0] = fmax(a, mx[0]);
    out[1] = fmin(b, mn[0]);
  }
}

// perm[i] = original row that ends in position i after applying ipiv in order.
__global__ void compose_perm(int64_t n, const int32_t *ipiv, int32_t *perm) {
  extern __shared__ int32_t p[];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) p[i] = (int32_t)i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int64_t i = 0; i < n; ++i) {
      const int32_t t = ipiv[i] - 1;
      if (t < i || t >= n) continue;  // not a pivot LU can produce: never index outside p
      const int32_t v = p[i];
      p[i] = p[t];
      p[t] = v;
    }
  }
  __syncthreads();
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) perm[i] = p[i];
}

// max that keeps a NaN (fmax would drop it): the norms below feed the
// backward-error test, which must fail on a NaN anywhere in x or r
__device__ __forceinline__ double nan_max(double a, double b) { return (b > a || b != b) ? b : a; }

// Per right-hand side: out[c] = max_i |v[i, c]| (one CTA per column).
__global__ void col_absmax(int64_t n, const double *__restrict__ v, int64_t ldv, double *out) {
  __shared__ double red[32];
  const int c = blockIdx.x;
  double m = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = nan_max(m, fabs(v[i + c * ldv]));
  for (int off = 16; off > 0; off >>= 1) m = nan_max(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mm = nan_max(mm, red[w]);
    out[c] = mm;
  }
}

__global__ void max_of(int64_t n, const double *v, double *out) {
  __shared__ double red[32];
  double m = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = nan_max(m, v[i]);
  for (int off = 16; off > 0; off >>= 1) m = nan_max(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mm = nan_max(mm, red[w]);
    *out = mm;
  }
}

// y[i, c] = fl32(pre[p] r[p, c] / rscale[c]), p = perm[i] (pre: the row
// scale of a Cholesky's D A D, or none)
template <typename T>
__global__ void permute_scale_down(int64_t n, int nrhs, const double *__restrict__ r, int64_t ldr,
                                   const int32_t *perm, const double *rscale, T *__restrict__ y, const double *pre) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int64_t i = e % n, c = e / n;
  const double s = rscale[c];
  const int64_t p = perm[i];
  const double v = pre != nullptr ? r[p + c * ldr] * pre[p] : r[p + c * ldr];
  y[i + c * n] = s > 0.0 ? (T)(v / s) : T(0);
}

// x[i, c] += S_i * rscale[c] * y[i, c]   (or x = ... when assign); S_i is
// the column scale of the LU's 64-column block, or the row scale postrow[i]
// of a Cholesky
template <typename T>
__global__ void update_x(int64_t n, int nrhs, const T *__restrict__ y, const double *scale, const double *rscale,
                         double *__restrict__ x, int64_t ldx, int assign, const double *postrow) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int64_t i = e % n, c = e / n;
  const double d = (double)y[i + c * n] * (postrow != nullptr ? postrow[i] : scale[i / TB]) * rscale[c];
  double *p = x + i + c * ldx;
  *p = assign ? d : *p + d;
}

__global__ void copy_cols(int64_t n, int nrhs, const double *__restrict__ src, int64_t lds, double *__restrict__ dst,
                          int64_t ldd) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int64_t i = e % n, c = e / n;
  dst[i + c * ldd] = src[i + c * lds];
}

// Symmetric scaling of an SPD matrix: d_i = 2^-k with a_ii 2^-2k in
// [0.5, 2), exact, so D A D has an O(1) diagonal.  A diagonal entry that is
// not positive and finite gets d_i = 1 (the Cholesky then stops at it).
__global__ void sym_scale(int64_t n, const double *__restrict__ A, int64_t lda, double *d) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = A[i + i * lda];
  if (!(a > 0.0) || !isfinite(a)) {
    d[i] = 1.0;
    return;
  }
  int e = 0;
  frexp(a, &e);
  d[i] = ldexp(1.0, -(e >> 1));
}

// W = fl(D A D), lower triangle only (the Cholesky reads no other part).
template <typename T>
__global__ void convert_sym_lower(int64_t n, const double *__restrict__ A, int64_t lda, const double *d,
                                  T *__restrict__ W, int64_t ldw) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int64_t i = e % n, j = e / n;
  if (i < j) return;
  W[i + j * ldw] = (T)(A[i + j * lda] * d[i] * d[j]);
}

__global__ void iota_perm(int64_t n, int32_t *perm) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) perm[i] = (int32_t)i;
}

// Inverses of the 64x64 diagonal blocks of L (unit lower) and U, once per
// factorisation: block b -> Dl[b], Du[b] (column-major 64x64).  A thread per
// column of the inverse, substitution down (L) or up (U) the block.
template <typename T>
__global__ void __launch_bounds__(64)
diag_block_inverses(int64_t n, const T *__restrict__ W, int64_t ldw, T *Dl, T *Du) {
  __shared__ T B[TB][TB + 1];
  const int64_t k0 = (int64_t)blockIdx.x * TB;
  const int kb = (int)imin(TB, n - k0);
  // the whole tile is written: the substitutions below multiply entries
  // outside the kb x kb block by zeros, and 0 * (stale NaN) would be NaN
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e % TB, c = e / TB;
    B[r][c] = (r < kb && c < kb) ? W[(k0 + r) + (k0 + c) * ldw] : T(0);
  }
  __syncthreads();
  const int j = threadIdx.x;
  T *L = Dl + (int64_t)blockIdx.x * TB * TB, *U = Du + (int64_t)blockIdx.x * TB * TB;
  if (j >= TB) return;
  T x[TB];
#pragma unroll
  for (int i = 0; i < TB; ++i) {  // L x = e_j (unit diagonal)
    T t = (i == j) ? T(1) : T(0);
#pragma unroll
    for (int k = 0; k < i; ++k) t = fmaT(-B[i][k], x[k], t);
    x[i] = (i < kb) ? t : T(0);
  }
#pragma unroll
  for (int i = 0; i < TB; ++i) L[i + j * TB] = (j < kb) ? x[i] : T(0);
#pragma unroll
  for (int ii = 0; ii < TB; ++ii) {  // U x = e_j
    const int i = TB - 1 - ii;
    T t = (i == j) ? T(1) : T(0);
#pragma unroll
    for (int k = i + 1; k < TB; ++k) t = fmaT(-B[i][k], x[k], t);
    x[i] = (i < kb && j < kb) ? t / B[i][i] : T(0);
  }
#pragma unroll
  for (int i = 0; i < TB; ++i) U[i + j * TB] = x[i];
}

__device__ __forceinline__ int ld_acquire(const int32_t *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int32_t *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Blocked triangular solve with nrhs <= 32 right-hand sides (n x nrhs, ld n)
// in ONE launch, as a dataflow over the 64-row blocks.  LOWER: unit-lower L,
// blocks solved top to bottom; else U, bottom to top.  CTAs run in clusters
// of TCL: each cluster takes the next TCL blocks in solve order from an
// atomic ticket, so it only ever waits for blocks held by clusters that
// started before it (no co-residency assumption beyond the cluster's own).
// A solved block is published as 64-bit words (value bits, launch epoch):
// a reader spins on the words themselves, so one round trip to L2 both
// signals and delivers a block, and a writer needs no release fence (each
// word is written atomically and carries its own epoch).  Inside a cluster
// the block also goes straight to the shared memory of the next TNP CTAs
// (asynchronous remote stores completing on the receiver's mbarrier), so
// that a link between neighbours costs a shared-memory push, not an L2
// round trip.
// Block blk at position t in solve order folds in the blocks solved before
// its last TNP predecessors as they appear,
//   acc -= T[blk, k] x_k              (the tiles and words of the next two
//                                      blocks in flight during a product)
// and then, with c = Dinv acc formed before any predecessor is needed,
//   x_blk = c - sum_{d=1..TNP} C_d x_{t-d},   C_d = Dinv T[blk, t-d]
// (C_d precomputed per factorisation, bulk-copied into shared memory with
// Dinv at launch).  Predecessors pushed by the CTAs before it in the cluster
// (d <= rank) enter from its shared memory; those of an earlier cluster from
// their words, requested two ahead.  The chain between neighbours of a
// cluster is then one 64 x 64 product and a push; only a cluster's first
// block waits on an L2 round trip for the block before it.  Waits are
// bounded: on expiry *err is set (the host fails the solve) and the CTA goes
// on, so that every later wait still ends.
constexpr int TCL = 8;  // blocks (CTAs) per cluster of the FP32 solve
constexpr int TNP = 6;  // predecessors coupled through C_d

// bytes from global memory into this CTA's shared memory, completing on bar
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   sm100::smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(sm100::smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_word(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// C_d[b] = Dinv_b T[b, k] (column-major 64 x 64), k the block d places
// before b in solve order (d = blockIdx.y + 1): L[b, b - d] (lower),
// U[b, b + d] (upper).  C holds C_d for all blocks at C + ((d-1) nb + b) 4096.
template <bool LOWER>
__global__ void __launch_bounds__(256)
couple_blocks(int64_t n, const float *__restrict__ W, int64_t ldw, const float *__restrict__ Dinv, float *C) {
  __shared__ float D[TB][TB + 1], T[TB][TB + 1];
  const int nb = (int)cdiv(n, TB);
  const int b = blockIdx.x, d = (int)blockIdx.y + 1;
  float *outp = C + ((int64_t)(d - 1) * nb + b) * TB * TB;
  const int k = LOWER ? b - d : b + d;
  if (k < 0 || k >= nb) return;
  const int64_t i0 = (int64_t)b * TB, k0 = (int64_t)k * TB;
  const int kb = (int)imin(TB, n - i0), kbk = (int)imin(TB, n - k0);
  for (int e = threadIdx.x; e < TB * TB; e += 256) {
    const int r = e % TB, c = e / TB;
    D[r][c] = Dinv[(int64_t)b * TB * TB + e];
    T[r][c] = (r < kb && c < kbk) ? W[(i0 + r) + (k0 + c) * ldw] : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < TB * TB; e += 256) {
    const int r = e % TB, c = e / TB;
    float v = 0.f;
#pragma unroll 16
    for (int q = 0; q < TB; ++q) v = fmaf(D[r][q], T[q][c], v);
    outp[e] = v;
  }
}

// Sums of products A X (A a 64 x 64 operand, A[kk][r] = A(r, kk); X a
// 64 x (4 RH) block, X[kk][c]) formed in registers, then subtracted at once
// from the outputs a thread owns (row r, right-hand sides g RH ..).
// RH = 4 (16 right-hand sides): K is split in four; thread (ks, rg, cg) =
// (tid / 64, tid % 16, tid / 16 % 4) accumulates the 4 x 4 tile of rows
// 4 rg.., right-hand sides 4 cg.. over kk in [16 ks, 16 ks + 16) from two
// 16-byte loads and 16 independent FMAs a step; subtract_from meets the
// partials in red (red[(ks 16 + c) 64 + r], slices summed in order) behind
// one barrier, so several products added in turn pay for one reduction.
// Other RH: thread (r, g) runs the sums itself (two partial sums, even and
// odd kk).
template <int RH>
struct ProductSums {
  static constexpr int NP = RH == 4 ? 16 : RH;
  float p[NP];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < NP; ++i) p[i] = 0.f;
  }
  __device__ __forceinline__ void add(const float (*A)[TB], const float (*X)[4 * RH], int r, int g) {
    if constexpr (RH == 4) {
      const int tid = threadIdx.x, ks = tid >> 6, rg = tid & 15, cg = (tid >> 4) & 3;
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int kk = ks * 16 + q;
        const float4 a = *reinterpret_cast<const float4 *>(&A[kk][4 * rg]);
        const float4 x = *reinterpret_cast<const float4 *>(&X[kk][4 * cg]);
        const float av[4] = {a.x, a.y, a.z, a.w}, xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) p[4 * i + j] = fmaf(av[i], xv[j], p[4 * i + j]);
      }
    } else {
      float q2[2][RH];
#pragma unroll
      for (int c = 0; c < RH; ++c) q2[0][c] = q2[1][c] = 0.f;
#pragma unroll 8
      for (int kk = 0; kk < TB; ++kk) {
        const float a = A[kk][r];
#pragma unroll
        for (int c = 0; c < RH; c += 4) {
          const float4 x = *reinterpret_cast<const float4 *>(&X[kk][g * RH + c]);
          float *q = q2[kk & 1];
          q[c] = fmaf(a, x.x, q[c]);
          q[c + 1] = fmaf(a, x.y, q[c + 1]);
          q[c + 2] = fmaf(a, x.z, q[c + 2]);
          q[c + 3] = fmaf(a, x.w, q[c + 3]);
        }
      }
#pragma unroll
      for (int c = 0; c < RH; ++c) p[c] += q2[0][c] + q2[1][c];
    }
  }
  // acc -= the sums added since zero(), which this also does again.  RH = 4:
  // the caller has synchronised the CTA since red was last read.
  __device__ __forceinline__ void subtract_from(float (&acc)[RH], float *red, int r, int g) {
    if constexpr (RH == 4) {
      const int tid = threadIdx.x, ks = tid >> 6, rg = tid & 15, cg = (tid >> 4) & 3;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        *reinterpret_cast<float4 *>(&red[(ks * 16 + 4 * cg + j) * TB + 4 * rg]) =
            make_float4(p[j], p[4 + j], p[8 + j], p[12 + j]);
      __syncthreads();
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int col = 4 * g + c;
        acc[c] -= ((red[col * TB + r] + red[(16 + col) * TB + r]) + red[(32 + col) * TB + r]) +
                  red[(48 + col) * TB + r];
      }
    } else {
#pragma unroll
      for (int c = 0; c < RH; ++c) acc[c] -= p[c];
    }
    zero();
  }
};

// acc -= A X, one product (the caller has synchronised the CTA since red was last read)
template <int RH>
__device__ __forceinline__ void block_product(float (&acc)[RH], const float (*A)[TB], const float (*X)[4 * RH],
                                              float *red, int r, int g) {
  ProductSums<RH> s;
  s.zero();
  s.add(A, X, r, g);
  s.subtract_from(acc, red, r, g);
}

// A thread's share of one published block's words (row tid % 64, the RH
// right-hand sides of group tid / 64): loaded together, then polled again
// together (all those not yet published) until every one carries this
// launch's epoch: one L2 round trip per pass, not one per word.  A warp's
// loads of one right-hand side are 32 consecutive rows; its stores to X are
// 16 bytes a thread.
template <int RH>
struct BlockWords {
  unsigned long long w[RH];
  __device__ __forceinline__ bool need(int u, int kbk, int nrhs) const {
    return (int)(threadIdx.x % TB) < kbk && (int)(threadIdx.x / TB) * RH + u < nrhs;
  }
  __device__ __forceinline__ const unsigned long long *at(const unsigned long long *xw, int64_t n, int64_t k0,
                                                          int u) const {
    return xw + (k0 + threadIdx.x % TB) + (int64_t)((threadIdx.x / TB) * RH + u) * n;
  }
  __device__ __forceinline__ void load(const unsigned long long *xw, int64_t n, int nrhs, int64_t k0, int kbk) {
#pragma unroll
    for (int u = 0; u < RH; ++u) w[u] = need(u, kbk, nrhs) ? ld_word(at(xw, n, k0, u)) : 0ull;
  }
  // requests again the words that did not yet carry epoch when they came back
  __device__ __forceinline__ void refresh(const unsigned long long *xw, int64_t n, int nrhs, int64_t k0, int kbk,
                                          uint32_t epoch) {
#pragma unroll
    for (int u = 0; u < RH; ++u)
      if (need(u, kbk, nrhs) && (uint32_t)(w[u] >> 32) != epoch) w[u] = ld_word(at(xw, n, k0, u));
  }
  // spins until the words carry epoch, then writes them to X[kk][c]
  __device__ __forceinline__ void take(const unsigned long long *xw, int64_t n, int nrhs, int64_t k0, int kbk,
                                       uint32_t epoch, float (*X)[4 * RH], int32_t *err) {
    for (int polls = 0;; ++polls) {
      bool done = true;
#pragma unroll
      for (int u = 0; u < RH; ++u) done = done && (!need(u, kbk, nrhs) || (uint32_t)(w[u] >> 32) == epoch);
      if (done) break;
      if (polls >= (1 << 20)) {
        atomicExch(err, 3);
        break;
      }
#pragma unroll
      for (int u = 0; u < RH; ++u)
        if (need(u, kbk, nrhs) && (uint32_t)(w[u] >> 32) != epoch) w[u] = ld_word(at(xw, n, k0, u));
    }
    float *row = &X[threadIdx.x % TB][(threadIdx.x / TB) * RH];
#pragma unroll
    for (int u = 0; u < RH; u += 4) {
      float4 v;
      v.x = need(u, kbk, nrhs) ? __uint_as_float((uint32_t)w[u]) : 0.f;
      v.y = need(u + 1, kbk, nrhs) ? __uint_as_float((uint32_t)w[u + 1]) : 0.f;
      v.z = need(u + 2, kbk, nrhs) ? __uint_as_float((uint32_t)w[u + 2]) : 0.f;
      v.w = need(u + 3, kbk, nrhs) ? __uint_as_float((uint32_t)w[u + 3]) : 0.f;
      *reinterpret_cast<float4 *>(row + u) = v;
    }
  }
};

// dynamic shared memory of trsv_words: the operands Dinv, C_1..C_TNP; two
// fold tiles; two fold blocks; the TNP pushed predecessors; (RH = 4) the
// products' reduction buffer
template <int RH>
constexpr size_t trsv_words_smem() {
  return sizeof(float) * ((size_t)(TNP + 1) * TB * TB + 2 * TB * TB + (2 + TNP) * TB * 4 * RH +
                          (RH == 4 ? 4 * 16 * TB : 0));
}
// one CTA per SM: dynamic plus static (barriers, ticket) within the 227 KB a CTA may hold
static_assert(trsv_words_smem<4>() + 128 <= 227 * 1024, "trsv_words<RH = 4> shared memory");
static_assert(trsv_words_smem<8>() + 128 <= 227 * 1024, "trsv_words<RH = 8> shared memory");

template <bool LOWER, int RH>
__global__ void __launch_bounds__(256)
trsv_words(int64_t n, int nrhs, const float *__restrict__ W, int64_t ldw, const float *__restrict__ Dinv,
           const float *__restrict__ C, const float *__restrict__ y, float *out, unsigned long long *xw,
           int32_t *ticket, uint32_t epoch, int32_t *err) {
  extern __shared__ __align__(128) float tsm[];
  using Tile = float[TB][TB];      // Tile[kk][r] = operand(r, kk), the column-major 64 x 64 block
  using Blk = float[TB][4 * RH];   // Blk[kk][c]
  Tile *Op = reinterpret_cast<Tile *>(tsm);          // Op[0] = Dinv, Op[d] = C_d
  Tile *A = Op + TNP + 1;                            // fold tiles (alternating)
  Blk *X = reinterpret_cast<Blk *>(A + 2);           // fold blocks (alternating)
  Blk *Xp = X + 2;                                   // Xp[d-1]: the block d before, pushed by its CTA
  float *red = reinterpret_cast<float *>(Xp + TNP);  // (RH = 4) partial products
  __shared__ __align__(8) uint64_t xbar[TNP];        // complete when those pushes have landed
  __shared__ __align__(8) uint64_t obar;             // complete when the operands have landed
  __shared__ int sb;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const int nb = (int)cdiv(n, TB);
  constexpr uint32_t XBYTES = sizeof(Blk), OBYTES = sizeof(Tile);
  if (tid == 0) {
#pragma unroll
    for (int d = 0; d < TNP; ++d) sm100::mbar_init(&xbar[d], 1);
    sm100::mbar_init(&obar, 1);
    sm100::fence_mbar_init();
    if (rank == 0) sb = atomicAdd(ticket, 1);
  }
  cluster.sync();  // every CTA's barriers initialised; the cluster's ticket taken
  if (tid == 0 && rank != 0) sb = *cluster.map_shared_rank(&sb, 0);
  __syncthreads();
  const int t = sb * TCL + rank;  // position in solve order
  const bool live = t < nb;
  const int b = LOWER ? t : nb - 1 - t;
  const int kc = t < TNP ? t : TNP;  // predecessors coupled through C_d
  if (tid == 0 && live) {
    // the pushes from the CTAs before, inside the cluster; the operands
#pragma unroll
    for (int d = 1; d <= TNP; ++d)
      if (rank >= d) sm100::mbar_arrive_expect_tx(&xbar[d - 1], XBYTES);
    const int nops = 1 + kc;
    sm100::mbar_arrive_expect_tx(&obar, OBYTES * nops);
    bulk_load(Op[0], Dinv + (int64_t)b * TB * TB, OBYTES, &obar);
    for (int d = 1; d < nops; ++d) bulk_load(Op[d], C + ((int64_t)(d - 1) * nb + b) * TB * TB, OBYTES, &obar);
  }
  const int64_t i0 = (int64_t)b * TB;
  const int kb = live ? (int)imin(TB, n - i0) : 0;
  const int r = tid & (TB - 1), g = tid >> 6;  // row of the block, right-hand-side group (4 groups of RH)
  if (live) {
    float acc[RH];
#pragma unroll
    for (int c = 0; c < RH; ++c) {
      const int cc = g * RH + c;
      acc[c] = (cc < nrhs && r < kb) ? y[i0 + r + (int64_t)cc * n] : 0.f;
    }
    constexpr int PER = TB * TB / 256;
    // the blocks solved before the coupled predecessors; each block's tile
    // and words are requested two folds before its own
    const int nf = t - kc;
    auto tile_load = [&](float (&lv)[PER], int sidx) {
      const int64_t k0 = (int64_t)(LOWER ? sidx : nb - 1 - sidx) * TB;
      const int kbk = (int)imin(TB, n - k0);
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int e = tid + 256 * q;
        const int rr = e % TB, kk = e / TB;
        lv[q] = (rr < kb && kk < kbk) ? W[(i0 + rr) + (k0 + kk) * ldw] : 0.f;
      }
    };
    auto words_load = [&](BlockWords<RH> &w, int sidx) {
      const int64_t k0 = (int64_t)(LOWER ? sidx : nb - 1 - sidx) * TB;
      w.load(xw, n, nrhs, k0, (int)imin(TB, n - k0));
    };
    // one fold: block sidx's tile and words (in lvs, wds) into A, X[sidx & 1];
    // block sidx + 2's requested into the same registers before the product
    auto fold = [&](float(&lvs)[PER], BlockWords<RH> &wds, int sidx) {
      const int64_t k0 = (int64_t)(LOWER ? sidx : nb - 1 - sidx) * TB;
      const int kbk = (int)imin(TB, n - k0);
      const int h = sidx & 1;
      wds.take(xw, n, nrhs, k0, kbk, epoch, X[h], err);
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int e = tid + 256 * q;
        A[h][e / TB][e % TB] = lvs[q];
      }
      if (sidx + 2 < nf) {
        tile_load(lvs, sidx + 2);
        words_load(wds, sidx + 2);
      }
      __syncthreads();  // (also: every thread is past the product that last read A[h], X[h])
      block_product<RH>(acc, A[h], X[h], red, r, g);
    };
    float lv0[PER], lv1[PER];
    BlockWords<RH> wd, wd1;
    if (nf > 0) {
      tile_load(lv0, 0);
      words_load(wd, 0);
    }
    if (nf > 1) {
      tile_load(lv1, 1);
      words_load(wd1, 1);
    }
    for (int sidx = 0; sidx < nf; sidx += 2) {
      fold(lv0, wd, sidx);
      if (sidx + 1 < nf) fold(lv1, wd1, sidx + 1);
    }
    // the coupled predecessors of an earlier cluster (d > rank: no push comes
    // for them) are taken from their words into their unused push slots,
    // Xp[d-1], furthest first; like the folds', their words are requested
    // two ahead (the first two before the Dinv product)
    const int nl = kc > rank ? kc - rank : 0;  // d = kc, kc - 1, ..., rank + 1
    float cv[RH];                              // this block's solution
    // sum_d C_d x_{t-d}, subtracted from cv after the last coupling (at most
    // TNP products share one reduction; the folds, up to n/64 of them, each
    // take their own, which keeps their FP32 sums short)
    ProductSums<RH> csum;
    csum.zero();
    auto l2_load = [&](BlockWords<RH> &w, int i) {
      const int64_t p0 = (int64_t)(LOWER ? b - (kc - i) : b + (kc - i)) * TB;
      w.load(xw, n, nrhs, p0, (int)imin(TB, n - p0));
    };
    // (the next one's words, requested before this one's wait, are requested
    // again where they came back stale: the nearest predecessors are published
    // only about then)
    auto l2_couple = [&](BlockWords<RH> &w, BlockWords<RH> &next, int i) {
      const int d = kc - i;
      const int64_t p0 = (int64_t)(LOWER ? b - d : b + d) * TB;
      w.take(xw, n, nrhs, p0, (int)imin(TB, n - p0), epoch, Xp[d - 1], err);
      if (i + 2 < nl) l2_load(w, i + 2);
      if (i + 1 < nl) {
        const int64_t p1 = (int64_t)(LOWER ? b - d + 1 : b + d - 1) * TB;
        next.refresh(xw, n, nrhs, p1, (int)imin(TB, n - p1), epoch);
      }
      __syncthreads();
      csum.add(Op[d], Xp[d - 1], r, g);
    };
    if (nl > 0) l2_load(wd, 0);
    if (nl > 1) l2_load(wd1, 1);
    // c = Dinv acc: acc into X[0] as a 64 x (4 RH) operand
    __syncthreads();  // every thread is past the last fold's product
#pragma unroll
    for (int c = 0; c < RH; ++c) X[0][r][g * RH + c] = acc[c];
    if (!__syncthreads_and(sm100::bounded_wait(&obar, 0u)) && tid == 0) atomicExch(err, 3);
#pragma unroll
    for (int c = 0; c < RH; ++c) cv[c] = 0.f;
    block_product<RH>(cv, Op[0], X[0], red, r, g);  // cv = -Dinv acc
#pragma unroll
    for (int c = 0; c < RH; ++c) cv[c] = -cv[c];
    // x = c - sum_d C_d x_{t-d}: first the predecessors from words, then the
    // pushed ones, furthest first
    for (int i = 0; i < nl; i += 2) {
      l2_couple(wd, wd1, i);
      if (i + 1 < nl) l2_couple(wd1, wd, i + 1);
    }
#pragma unroll
    for (int d = TNP; d >= 1; --d) {
      if (d > kc || d > rank) continue;
      if (!__syncthreads_and(sm100::bounded_wait(&xbar[d - 1], 0u)) && tid == 0) atomicExch(err, 3);
      csum.add(Op[d], Xp[d - 1], r, g);
    }
    // (each coupling above passed a barrier after the Dinv product read red)
    if (kc > 0) csum.subtract_from(cv, red, r, g);
    // to the next TNP CTAs of the cluster (their Xp[d-1]): each thread stores
    // its row's values straight from registers (st.async, completing on the
    // receiver's mbarrier); then the words, for the CTAs of later clusters
#pragma unroll
    for (int d = 1; d <= TNP; ++d) {
      if (rank + d >= TCL || t + d >= nb) break;
      const uint32_t bar = sm100::cluster_addr(&xbar[d - 1], rank + d);
#pragma unroll
      for (int c = 0; c < RH; c += 4)
        sm100::st_async4(sm100::cluster_addr(&Xp[d - 1][r][g * RH + c], rank + d), __float_as_uint(cv[c]),
                         __float_as_uint(cv[c + 1]), __float_as_uint(cv[c + 2]), __float_as_uint(cv[c + 3]), bar);
    }
    if (r < kb) {
#pragma unroll
      for (int c = 0; c < RH; ++c) {
        const int cc = g * RH + c;
        if (cc >= nrhs) continue;
        const int64_t idx = i0 + r + (int64_t)cc * n;
        st_word(xw + idx, ((unsigned long long)epoch << 32) | __float_as_uint(cv[c]));
        out[idx] = cv[c];
      }
    }
  }
  cluster.sync();  // no CTA leaves while one before may still push into it
}

// The FP64 form of the same dataflow, for the FP64-storage factor.  GB300's
// FP64 pipe retires about two FMAs per clock per SM, so one CTA per block
// would make each block's work a long serial chain; here a CTA of 64
// threads owns one (block, right-hand side) pair: thread r keeps row r's
// accumulator, prefetches its row of each L (U) tile before waiting for the
// tile's solved block, and the 64 x 64 diagonal inverse finishes the block.
// Flags are per (block, right-hand side); tickets run block-major, so a CTA
// again only waits for CTAs that started before it.
template <bool LOWER>
__global__ void __launch_bounds__(64)
trsv_dataflow64(int64_t n, int nrhs, const double *__restrict__ W, int64_t ldw, const double *__restrict__ Dinv,
                const double *__restrict__ y, double *out, int32_t *flags, int32_t *ticket, int32_t epoch,
                int32_t *err) {
  __shared__ double xs[TB];
  __shared__ int sb;
  const int r = threadIdx.x;
  const int nb = (int)((n + TB - 1) / TB);
  if (r == 0) sb = atomicAdd(ticket, 1);
  __syncthreads();
  const int sidx = sb / nrhs, c = sb % nrhs;  // position in solve order, right-hand side
  const int b = LOWER ? sidx : nb - 1 - sidx;
  const int64_t i0 = (int64_t)b * TB;
  const int kb = (int)imin(TB, n - i0);
  double acc = r < kb ? y[i0 + r + (int64_t)c * n] : 0.0;
  for (int q = 0; q < sidx; ++q) {
    const int k = LOWER ? q : nb - 1 - q;
    const int64_t k0 = (int64_t)k * TB;
    const int kbk = (int)imin(TB, n - k0);
    double lv[TB];
    const double *Lr = W + (i0 + (r < kb ? r : 0)) + k0 * ldw;
#pragma unroll
    for (int kk = 0; kk < TB; ++kk) lv[kk] = (r < kb && kk < kbk) ? Lr[(int64_t)kk * ldw] : 0.0;
    if (r == 0) {
      int polls = 0;
      while (ld_acquire(flags + (int64_t)k * MAXRHS + c) != epoch) {
        if (++polls > (1 << 21)) {
          atomicExch(err, 3);
          break;
        }
        __nanosleep(64);
      }
    }
    __syncthreads();
    xs[r] = r < kbk ? __ldcg(out + k0 + r + (int64_t)c * n) : 0.0;
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TB; ++kk) acc = fma(-lv[kk], xs[kk], acc);
    __syncthreads();
  }
  xs[r] = acc;
  __syncthreads();
  const double *D = Dinv + (int64_t)b * TB * TB;
  double v = 0.0;
#pragma unroll 8
  for (int kk = 0; kk < TB; ++kk) v = fma(D[r + kk * TB], xs[kk], v);
  if (r < kb) out[i0 + r + (int64_t)c * n] = v;
  __threadfence();
  __syncthreads();
  if (r == 0) st_release(flags + (int64_t)b * MAXRHS + c, epoch);
}

// Sequencing state of the dataflow solves: flags (one per 64-row block and
// right-hand side, zeroed once), the ticket, the wait-expiry flag and the
// launch epoch.
struct TrsvSync {
  int32_t *flags = nullptr, *ticket = nullptr, *err = nullptr;
  int32_t epoch = 0;
  unsigned long long *xw = nullptr;  // published blocks of the FP32 solves (value, epoch)
  // Dinv times the blocks 1..TNP places back in solve order, per 64-row block (lower, upper factor)
  const float *Cl = nullptr, *Cu = nullptr;
};

// y (right-hand sides) -> out (solution); y is not modified.
int trsv(cudaStream_t s, bool lower, int64_t n, int nrhs, const float *W, int64_t ldw, const float *Dinv,
         const float *y, float *out, TrsvSync &sync);
int trsv(cudaStream_t s, bool lower, int64_t n, int nrhs, const double *W, int64_t ldw, const double *Dinv,
         const double *y, double *out, TrsvSync &sync) {
  ProfScope prof(s, lower ? "trsv64_lower" : "trsv64_upper", (double)n * n * nrhs, 8.0 * (double)n * n / 2, 1);
  const unsigned grid = (unsigned)(cdiv(n, TB) * nrhs);
  const int32_t epoch = ++sync.epoch;
  BOLA_TRY_CUDA(cudaMemsetAsync(sync.ticket, 0, sizeof(int32_t), s));
  if (lower)
    trsv_dataflow64<true><<<grid, TB, 0, s>>>(n, nrhs, W, ldw, Dinv, y, out, sync.flags, sync.ticket, epoch, sync.err);
  else
    trsv_dataflow64<false><<<grid, TB, 0, s>>>(n, nrhs, W, ldw, Dinv, y, out, sync.flags, sync.ticket, epoch, sync.err);
  BOLA_CHECK_LAUNCH();
  return 0;
}
int trsv(cudaStream_t s, bool lower, int64_t n, int nrhs, const float *W, int64_t ldw, const float *Dinv,
         const float *y, float *out, TrsvSync &sync) {
  ProfScope prof(s, lower ? "trsv_lower" : "trsv_upper", (double)n * n * nrhs, 4.0 * (double)n * n / 2, 1);
  const unsigned nb = (unsigned)cdiv(n, TB);
  const uint32_t epoch = (uint32_t)++sync.epoch;
  BOLA_TRY_CUDA(cudaMemsetAsync(sync.ticket, 0, sizeof(int32_t), s));
  const float *C = lower ? sync.Cl : sync.Cu;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(cdiv(nb, TCL) * TCL));
  cfg.blockDim = dim3(256);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = TCL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
#define BOLA_TRSV(LW, RH)                                                                                    \
  do {                                                                                                       \
    static bool attr_set = false;                                                                            \
    if (!attr_set) {                                                                                         \
      BOLA_TRY_CUDA(cudaFuncSetAttribute(trsv_words<LW, RH>, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                         (int)trsv_words_smem<RH>()));                                       \
      if (TCL > 8)                                                                                           \
        BOLA_TRY_CUDA(                                                                                       \
            cudaFuncSetAttribute(trsv_words<LW, RH>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));    \
      attr_set = true;                                                                                       \
    }                                                                                                        \
    cfg.dynamicSmemBytes = trsv_words_smem<RH>();                                                            \
    BOLA_TRY_CUDA(cudaLaunchKernelEx(&cfg, trsv_words<LW, RH>, n, nrhs, W, ldw, Dinv, C, y, out, sync.xw,    \
                                     sync.ticket, epoch, sync.err));                                         \
  } while (0)
  if (nrhs <= 16) {
    if (lower) BOLA_TRSV(true, 4);
    else BOLA_TRSV(false, 4);
  } else {
    if (lower) BOLA_TRSV(true, 8);
    else BOLA_TRSV(false, 8);
  }
#undef BOLA_TRSV
  BOLA_CHECK_LAUNCH();
  return 0;
}

// Dinv times the coupling blocks of the FP32 factor's L and U (once per factorisation).
int couple(cudaStream_t s, int64_t n, const float *W, int64_t ldw, const float *Dl, const float *Du, float *Cl,
           float *Cu) {
  ProfScope prof(s, "trsv_couple", 2.0 * TNP * 2 * (double)cdiv(n, TB) * TB * TB * TB, 0.0, 2);
  const unsigned nb = (unsigned)cdiv(n, TB);
  couple_blocks<true><<<dim3(nb, TNP), 256, 0, s>>>(n, W, ldw, Dl, Cl);
  couple_blocks<false><<<dim3(nb, TNP), 256, 0, s>>>(n, W, ldw, Du, Cu);
  BOLA_CHECK_LAUNCH();
  return 0;
}

// ---- GMRES-IR (flexible GMRES on A d = r, preconditioned by the LU) -------------
// Basis layout: V[(k * nrhs + c) * n + row] (column k of right-hand side c).
constexpr int GM_M = 24;  // restart length

// H[i + c * ldh] = <V_i,c , w_c> for i < kk (one CTA per (i, c), fixed-order reduction)
__global__ void gm_dots(int64_t n, int nrhs, const double *__restrict__ V, const double *__restrict__ w, double *H,
                        int ldh) {
  __shared__ double red[32];
  const int i = blockIdx.x, c = blockIdx.y;
  const double *v = V + ((int64_t)i * nrhs + c) * n;
  const double *ww = w + (int64_t)c * n;
  double acc = 0.0;
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) acc = fma(v[r], ww[r], acc);
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    H[i + c * ldh] = t;
  }
}

// w_c -= sum_{i<kk} V_i,c * H[i + c*ldh]
__global__ void gm_sub(int64_t n, int nrhs, int kk, const double *__restrict__ V, const double *__restrict__ H,
                       int ldh, double *w) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int64_t r = e % n;
  const int c = (int)(e / n);
  double acc = w[r + (int64_t)c * n];
  for (int i = 0; i < kk; ++i) acc = fma(-V[((int64_t)i * nrhs + c) * n + r], H[i + c * ldh], acc);
  w[r + (int64_t)c * n] = acc;
}

// out[c] = ||w_c||_2 (one CTA per column)
__global__ void gm_norm2(int64_t n, const double *__restrict__ w, double *out) {
  __shared__ double red[32];
  const int c = blockIdx.x;
  const double *ww = w + (int64_t)c * n;
  double acc = 0.0;
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) acc = fma(ww[r], ww[r], acc);
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    out[c] = sqrt(t);
  }
}

// V_k,c = w_c / nrm[c]  (zero when the norm is zero)
__global__ void gm_scale_into(int64_t n, int nrhs, const double *__restrict__ w, const double *nrm, double *Vk) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int c = (int)(e / n);
  const double s = nrm[c];
  Vk[e] = s > 0.0 ? w[e] / s : 0.0;
}

// x[r, c] += sum_{i<kk} Z_i,c[r] * y[i + c*ldy]
__global__ void gm_add_zy(int64_t n, int nrhs, int kk, const double *__restrict__ Z, const double *__restrict__ y,
                          int ldy, double *x, int64_t ldx) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int64_t r = e % n;
  const int c = (int)(e / n);
  double acc = 0.0;
  for (int i = 0; i < kk; ++i) acc = fma(Z[((int64_t)i * nrhs + c) * n + r], y[i + c * ldy], acc);
  x[r + c * ldx] += acc;
}

// Device workspace of one mixed solve, cached per device and grown on demand.
struct Workspace {
  int64_t n = 0, nrhs = 0, bytes = 0;
  int fkind = 2;        // factor kind of the current solve (3: FP64 W, y, z, Dl, Du)
  int64_t ldW = 0;      // leading dimension of W (FP64: padded to 32 for the TMA tiles)
  size_t wbytes = 0;    // bytes held by W
  void *W = nullptr;    // the working matrix, then its LU factors (FP32, or FP64 for kind 3)
  void *y = nullptr, *z = nullptr, *Dl = nullptr, *Du = nullptr;  // 8-byte elements, used as FP32 or FP64
  double *scale = nullptr, *r = nullptr, *d = nullptr, *norms = nullptr, *rowsum = nullptr;
  double *V = nullptr, *Z = nullptr, *H = nullptr;  // GMRES basis, preconditioned basis, Hessenberg column
  double *hn = nullptr;                              // per-column 2-norms (GMRES)
  int32_t *ipiv = nullptr, *perm = nullptr, *info = nullptr;
  bool chol = false;           // the current factor is a Cholesky (in LU form)
  bool split_kept = false;     // oz holds this call's A already (a solve handed on within one call)
  double *dscale = nullptr;    // its row scale D (W = D A D)
  void *dg = nullptr;          // scratch: the diagonal of L (8-byte elements)
  float *Mc = nullptr;         // FP32 factors: the couplings C_1..C_TNP of every block, lower then upper
  double *hpin = nullptr;      // pinned host staging of a sweep's norms and the wait-expiry flag
  TrsvSync ts;  // dataflow triangular solves
  MixedLU lu;
  OzMatrix oz;  // A's digit planes: the FP64-accurate products of the refinement
};

void ws_free(Workspace &w) {
  for (void *p : {(void *)w.W, (void *)w.y, (void *)w.z, (void *)w.Dl, (void *)w.Du, (void *)w.scale, (void *)w.r,
                  (void *)w.d, (void *)w.norms, (void *)w.rowsum, (void *)w.ipiv, (void *)w.perm, (void *)w.info,
                  (void *)w.V, (void *)w.Z, (void *)w.H, (void *)w.hn, (void *)w.ts.flags, (void *)w.ts.ticket,
                  (void *)w.dscale, w.dg, (void *)w.Mc, (void *)w.ts.xw})
    if (p) cudaFree(p);
  if (w.hpin) cudaFreeHost(w.hpin);
  w.hpin = nullptr;
  w.ts.flags = w.ts.ticket = w.ts.err = nullptr;
  w.lu.release(nullptr);
  w.oz.release();
  w.W = w.y = w.z = w.Dl = w.Du = nullptr;
  w.wbytes = 0;
  w.scale = w.r = w.d = w.norms = w.rowsum = w.V = w.Z = w.H = w.hn = nullptr;
  w.ipiv = w.perm = w.info = nullptr;
  w.dscale = nullptr;
  w.dg = nullptr;
  w.Mc = nullptr;
  w.ts.xw = nullptr;
  w.ts.Cl = w.ts.Cu = nullptr;
  w.n = w.nrhs = w.bytes = 0;
}

int ws_reserve(Workspace &w, int64_t n, int64_t nrhs, int kind, cudaStream_t s) {
  const int64_t n_req = n;  // the factorisation size; buffers may be larger
  if (n > w.n || nrhs > w.nrhs) {
    const int64_t nn = imax(n, w.n), rr = imax(nrhs, w.nrhs);
    w.lu.release(s);  // stream-ordered; the LU keeps its streams and events
    ws_free(w);
    n = nn;
    nrhs = rr;
    int64_t bytes = 0;
    auto alloc = [&](auto **p, size_t sz) -> int {
      bytes += (int64_t)sz;
      return cudaMalloc(reinterpret_cast<void **>(p), sz) == cudaSuccess ? 0 : fail(BOLA_ERR_CUDA, "mixed: out of memory");
    };
    w.wbytes = (size_t)(kind == 3 ? cdiv(n, 32) * 32 : n) * n * (kind == 3 ? 8 : 4);
    BOLA_TRY(alloc(&w.W, w.wbytes));
    BOLA_TRY(alloc(&w.y, sizeof(double) * n * nrhs));
    BOLA_TRY(alloc(&w.z, sizeof(double) * n * nrhs));
    BOLA_TRY(alloc(&w.Dl, sizeof(double) * cdiv(n, TB) * TB * TB));
    BOLA_TRY(alloc(&w.Du, sizeof(double) * cdiv(n, TB) * TB * TB));
    BOLA_TRY(alloc(&w.scale, sizeof(double) * cdiv(n, TB)));
    BOLA_TRY(alloc(&w.r, sizeof(double) * n * nrhs));
    BOLA_TRY(alloc(&w.d, sizeof(double) * n * nrhs));
    BOLA_TRY(alloc(&w.norms, sizeof(double) * 6 * MAXRHS));
    if (cudaMallocHost(reinterpret_cast<void **>(&w.hpin), sizeof(double) * (3 * MAXRHS + 2)) != cudaSuccess)
      return fail(BOLA_ERR_CUDA, "mixed: out of pinned host memory");
    BOLA_TRY(alloc(&w.rowsum, sizeof(double) * n));
    BOLA_TRY(alloc(&w.dscale, sizeof(double) * n));
    BOLA_TRY(alloc(&w.dg, sizeof(double) * n));
    BOLA_TRY(alloc(&w.ipiv, sizeof(int32_t) * n));
    BOLA_TRY(alloc(&w.perm, sizeof(int32_t) * n));
    BOLA_TRY(alloc(&w.info, sizeof(int32_t)));
    BOLA_TRY(alloc(&w.V, sizeof(double) * (GM_M + 1) * nrhs * n));
    BOLA_TRY(alloc(&w.Z, sizeof(double) * GM_M * nrhs * n));
    BOLA_TRY(alloc(&w.H, sizeof(double) * (GM_M + 2) * MAXRHS * 2));
    BOLA_TRY(alloc(&w.hn, sizeof(double) * MAXRHS));
    BOLA_TRY(alloc(&w.ts.flags, sizeof(int32_t) * cdiv(n, TB) * MAXRHS));
    BOLA_TRY(alloc(&w.ts.ticket, sizeof(int32_t) * 2));
    BOLA_TRY(alloc(&w.Mc, sizeof(float) * 2 * TNP * cdiv(n, TB) * TB * TB));
    BOLA_TRY(alloc(&w.ts.xw, sizeof(unsigned long long) * n * MAXRHS));
    // the published words start from epoch 0, which no launch uses
    BOLA_TRY_CUDA(cudaMemset(w.ts.xw, 0, sizeof(unsigned long long) * n * MAXRHS));
    w.ts.Cl = w.Mc;
    w.ts.Cu = w.Mc + TNP * cdiv(n, TB) * TB * TB;
    w.ts.err = w.ts.ticket + 1;
    BOLA_TRY_CUDA(cudaMemset(w.ts.flags, 0, sizeof(int32_t) * cdiv(n, TB) * MAXRHS));
    BOLA_TRY_CUDA(cudaMemset(w.ts.ticket, 0, sizeof(int32_t) * 2));
    w.ts.epoch = 0;
    w.n = n;
    w.nrhs = nrhs;
    w.bytes = bytes + (int64_t)n * 64 * 4 * 4;  // plus the update operands of the LU
  }
  const size_t wneed = (size_t)(kind == 3 ? cdiv(n_req, 32) * 32 : n_req) * n_req * (kind == 3 ? 8 : 4);
  if (w.wbytes < wneed) {  // an FP64 factor in a workspace sized for FP32 ones
    cudaStreamSynchronize(s);
    cudaFree(w.W);
    w.W = nullptr;
    w.bytes -= (int64_t)w.wbytes;
    w.wbytes = 0;
    if (cudaMalloc(&w.W, wneed) != cudaSuccess) return fail(BOLA_ERR_CUDA, "mixed: out of memory");
    w.wbytes = wneed;
    w.bytes += (int64_t)wneed;
  }
  const int64_t oz_before = w.oz.bytes;
  BOLA_TRY(w.oz.reserve(n_req));
  w.bytes += w.oz.bytes - oz_before;
  return w.lu.reserve(n_req, kind, s);
}

std::mutex g_ws_mu;
Workspace g_ws[64];

// Low-precision correction: y = S U^-1 L^-1 P (r / rs) * rs, added to (or assigned into) x.
int correction(cudaStream_t s, Workspace &w, int64_t n, int nrhs, const double *r, int64_t ldr, const double *rs,
               double *x, int64_t ldx, bool assign) {
  const unsigned g = (unsigned)cdiv(n * nrhs, 256);
  if (w.fkind == 3) {
    double *y = static_cast<double *>(w.y), *z = static_cast<double *>(w.z);
    const double *W = static_cast<const double *>(w.W);
    permute_scale_down<double><<<g, 256, 0, s>>>(n, nrhs, r, ldr, w.perm, rs, y, w.chol ? w.dscale : nullptr);
    BOLA_CHECK_LAUNCH();
    BOLA_TRY(trsv(s, true, n, nrhs, W, w.ldW, static_cast<const double *>(w.Dl), y, z, w.ts));
    BOLA_TRY(trsv(s, false, n, nrhs, W, w.ldW, static_cast<const double *>(w.Du), z, y, w.ts));
    update_x<double><<<g, 256, 0, s>>>(n, nrhs, y, w.scale, rs, x, ldx, assign ? 1 : 0, w.chol ? w.dscale : nullptr);
  } else {
    float *y = static_cast<float *>(w.y), *z = static_cast<float *>(w.z);
    const float *W = static_cast<const float *>(w.W);
    permute_scale_down<float><<<g, 256, 0, s>>>(n, nrhs, r, ldr, w.perm, rs, y, w.chol ? w.dscale : nullptr);
    BOLA_CHECK_LAUNCH();
    BOLA_TRY(trsv(s, true, n, nrhs, W, n, static_cast<const float *>(w.Dl), y, z, w.ts));
    BOLA_TRY(trsv(s, false, n, nrhs, W, n, static_cast<const float *>(w.Du), z, y, w.ts));
    update_x<float><<<g, 256, 0, s>>>(n, nrhs, y, w.scale, rs, x, ldx, assign ? 1 : 0, w.chol ? w.dscale : nullptr);
  }
  BOLA_CHECK_LAUNCH();
  return 0;
}

// r = b - A x in FP64, then the backward error over all right-hand sides.
int residual_berr(cudaStream_t s, Workspace &w, int64_t n, int nr, const double *a, int64_t lda, const double *b,
                  int64_t ldb, const double *x, int64_t ldx, double *berr) {
  double *nrm = w.norms;
  {
    ProfScope prof(s, "mixed_residual", 2.0 * (double)n * n * nr, 2.0 * OZ_SA * (double)n * n, 4 * (int)cdiv(nr, 16) + 2);
    BOLA_TRY(w.oz.product(s, nr, x, ldx, b, ldb, w.r, n, w.ts.err));
    col_absmax<<<nr, 256, 0, s>>>(n, w.r, n, nrm);
    col_absmax<<<nr, 256, 0, s>>>(n, x, ldx, nrm + nr);
  }
  BOLA_CHECK_LAUNCH();
  // through the workspace's pinned staging: both reads are truly asynchronous
  const double *h = w.hpin;
  int32_t *terr_h = reinterpret_cast<int32_t *>(w.hpin + 3 * MAXRHS + 1);
  BOLA_TRY_CUDA(cudaMemcpyAsync(w.hpin, nrm, sizeof(double) * (3 * nr + 1), cudaMemcpyDeviceToHost, s));
  BOLA_TRY_CUDA(cudaMemcpyAsync(terr_h, w.ts.err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  BOLA_TRY_CUDA(cudaStreamSynchronize(s));
  const int32_t terr = *terr_h;
  if (terr != 0) {
    cudaMemsetAsync(w.ts.err, 0, sizeof(int32_t), s);
    return fail(BOLA_ERR_CUDA, "mixed: a bounded wait expired in the refinement (code %d)", terr);
  }
  double e = 0.0;
  for (int c = 0; c < nr; ++c) {
    const double den = h[3 * nr] * h[nr + c] + h[2 * nr + c];
    const double v = den > 0.0 ? h[c] / den : (h[c] > 0.0 ? INFINITY : 0.0);
    e = std::isnan(v) ? INFINITY : fmax(e, v);
  }
  *berr = e;
  return 0;
}

// One GMRES-IR step: flexible GMRES (restart GM_M) on A d = r for the residual
// in w.r, right-preconditioned by the low-precision LU (z = M^-1 v through
// the FP32 triangular solves), FP64 matrix products (the exact DGEMM) and
// classical Gram-Schmidt with one reorthogonalisation; then x += Z y.
// Each right-hand side runs its own Krylov process; they advance together.
int gmres_step(cudaStream_t s, Workspace &w, int64_t n, int nr, const double *a, int64_t lda, double *x,
               int64_t ldx, double inner_tol, int *inner_iters) {
  const int ldh = GM_M + 2;
  double *H1 = w.H, *H2 = w.H + ldh * MAXRHS;  // device Hessenberg columns (two CGS passes)
  double *beta_d = w.norms + 4 * MAXRHS;       // per-column max |v| for the FP32 scaling
  const unsigned g = (unsigned)cdiv(n * nr, 256);
  gm_norm2<<<nr, 256, 0, s>>>(n, w.r, w.hn);
  gm_scale_into<<<g, 256, 0, s>>>(n, nr, w.r, w.hn, w.V);
  BOLA_CHECK_LAUNCH();
  std::vector<double> beta(nr), hd(2 * ldh * MAXRHS), hnh(MAXRHS);
  BOLA_TRY_CUDA(cudaMemcpyAsync(beta.data(), w.hn, sizeof(double) * nr, cudaMemcpyDeviceToHost, s));
  BOLA_TRY_CUDA(cudaStreamSynchronize(s));
  // per right-hand side: R (upper, column-major ldh), Givens cs/sn, rhs gvec
  std::vector<double> R((size_t)ldh * GM_M * nr, 0.0), cs((size_t)GM_M * nr), sn((size_t)GM_M * nr),
      gv((size_t)ldh * nr, 0.0);
  for (int c = 0; c < nr; ++c) gv[(size_t)c * ldh] = beta[c];
  int kk = 0;
  for (int k = 0; k < GM_M; ++k) {
    double *Vk = w.V + (int64_t)k * nr * n, *Zk = w.Z + (int64_t)k * nr * n;
    col_absmax<<<nr, 256, 0, s>>>(n, Vk, n, beta_d);
    BOLA_CHECK_LAUNCH();
    BOLA_TRY(correction(s, w, n, nr, Vk, n, beta_d, Zk, n, true));
    {
      ProfScope prof(s, "gmres_matvec", 2.0 * (double)n * n * nr, 2.0 * OZ_SA * (double)n * n, 4 * (int)cdiv(nr, 16));
      BOLA_TRY(w.oz.product(s, nr, Zk, n, nullptr, 0, w.d, n, w.ts.err));
    }
    {
      ProfScope prof(s, "gmres_orth", 8.0 * (double)n * nr * (k + 1), 0.0, 6);
      gm_dots<<<dim3(k + 1, nr), 256, 0, s>>>(n, nr, w.V, w.d, H1, ldh);
      gm_sub<<<g, 256, 0, s>>>(n, nr, k + 1, w.V, H1, ldh, w.d);
      gm_dots<<<dim3(k + 1, nr), 256, 0, s>>>(n, nr, w.V, w.d, H2, ldh);
      gm_sub<<<g, 256, 0, s>>>(n, nr, k + 1, w.V, H2, ldh, w.d);
      gm_norm2<<<nr, 256, 0, s>>>(n, w.d, w.hn);
      gm_scale_into<<<g, 256, 0, s>>>(n, nr, w.d, w.hn, w.V + (int64_t)(k + 1) * nr * n);
    }
    BOLA_CHECK_LAUNCH();
    BOLA_TRY_CUDA(cudaMemcpyAsync(hd.data(), w.H, sizeof(double) * 2 * ldh * MAXRHS, cudaMemcpyDeviceToHost, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(hnh.data(), w.hn, sizeof(double) * nr, cudaMemcpyDeviceToHost, s));
    BOLA_TRY_CUDA(cudaStreamSynchronize(s));
    kk = k + 1;
    bool done = true;
    for (int c = 0; c < nr; ++c) {
      double *col = &R[((size_t)c * GM_M + k) * ldh];
      for (int i = 0; i <= k; ++i) col[i] = hd[i + c * ldh] + hd[ldh * MAXRHS + i + c * ldh];
      col[k + 1] = hnh[c];
      double *csc = &cs[(size_t)c * GM_M], *snc = &sn[(size_t)c * GM_M], *gc = &gv[(size_t)c * ldh];
      for (int i = 0; i < k; ++i) {  // previous rotations
        const double t = csc[i] * col[i] + snc[i] * col[i + 1];
        col[i + 1] = -snc[i] * col[i] + csc[i] * col[i + 1];
        col[i] = t;
      }
      const double den = hypot(col[k], col[k + 1]);
      csc[k] = den > 0.0 ? col[k] / den : 1.0;
      snc[k] = den > 0.0 ? col[k + 1] / den : 0.0;
      col[k] = den;
      col[k + 1] = 0.0;
      gc[k + 1] = -snc[k] * gc[k];
      gc[k] = csc[k] * gc[k];
      if (beta[c] > 0.0 && fabs(gc[k + 1]) > inner_tol * beta[c]) done = false;
    }
    if (done) break;
  }
  *inner_iters += kk;
  // y = R^-1 g per right-hand side, then x += Z y
  std::vector<double> y((size_t)ldh * MAXRHS, 0.0);
  for (int c = 0; c < nr; ++c) {
    if (!(beta[c] > 0.0)) continue;
    for (int i = kk - 1; i >= 0; --i) {
      double t = gv[(size_t)c * ldh + i];
      for (int j = i + 1; j < kk; ++j) t -= R[((size_t)c * GM_M + j) * ldh + i] * y[(size_t)c * ldh + j];
      const double d = R[((size_t)c * GM_M + i) * ldh + i];
      y[(size_t)c * ldh + i] = d != 0.0 ? t / d : 0.0;
    }
  }
  BOLA_TRY_CUDA(cudaMemcpyAsync(H2, y.data(), sizeof(double) * ldh * MAXRHS, cudaMemcpyHostToDevice, s));
  gm_add_zy<<<g, 256, 0, s>>>(n, nr, kk, w.Z, H2, ldh, x, ldx);
  BOLA_CHECK_LAUNCH();
  BOLA_TRY_CUDA(cudaStreamSynchronize(s));  // y lives on this host stack frame
  return 0;
}

}  // namespace
}  // namespace bola

using namespace bola;

namespace bola {
namespace {

int dgesv_mixed_ws(Workspace &w, bool chol, int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *b,
                   int64_t ldb, double *x, int64_t ldx, const bola_mixed_opts *opts, bola_mixed_info *out,
                   cudaStream_t s);

}  // namespace
}  // namespace bola

extern "C" int bola_dgesv_mixed(int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *b, int64_t ldb,
                                double *x, int64_t ldx, const bola_mixed_opts *opts, bola_mixed_info *out,
                                bola_stream_t stream) {
  int dev = 0;
  BOLA_TRY_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_ws_mu);
  return dgesv_mixed_ws(g_ws[dev & 63], false, n, nrhs, a, lda, b, ldb, x, ldx, opts, out, (cudaStream_t)stream);
}

extern "C" int bola_dposv_mixed(int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *b, int64_t ldb,
                                double *x, int64_t ldx, const bola_mixed_opts *opts, bola_mixed_info *out,
                                bola_stream_t stream) {
  int dev = 0;
  BOLA_TRY_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_ws_mu);
  return dgesv_mixed_ws(g_ws[dev & 63], true, n, nrhs, a, lda, b, ldb, x, ldx, opts, out, (cudaStream_t)stream);
}

extern "C" int bola_dposv_mixed_ctx(bola_mixed_ctx ctx, int64_t n, int64_t nrhs, const double *a, int64_t lda,
                                    const double *b, int64_t ldb, double *x, int64_t ldx,
                                    const bola_mixed_opts *opts, bola_mixed_info *out, bola_stream_t stream) {
  Workspace *w = reinterpret_cast<Workspace *>(ctx);
  if (!w) return -1;
  return dgesv_mixed_ws(*w, true, n, nrhs, a, lda, b, ldb, x, ldx, opts, out, (cudaStream_t)stream);
}

extern "C" int bola_mixed_ctx_create(bola_mixed_ctx *ctx) {
  if (!ctx) return -1;
  *ctx = reinterpret_cast<bola_mixed_ctx>(new Workspace());
  return 0;
}

extern "C" int bola_mixed_ctx_destroy(bola_mixed_ctx ctx) {
  Workspace *w = reinterpret_cast<Workspace *>(ctx);
  if (!w) return 0;
  cudaDeviceSynchronize();
  ws_free(*w);
  w->lu.destroy();
  delete w;
  return 0;
}

extern "C" int64_t bola_mixed_ctx_bytes(bola_mixed_ctx ctx) {
  Workspace *w = reinterpret_cast<Workspace *>(ctx);
  return w ? w->bytes : 0;
}

extern "C" int bola_dgesv_mixed_ctx(bola_mixed_ctx ctx, int64_t n, int64_t nrhs, const double *a, int64_t lda,
                                    const double *b, int64_t ldb, double *x, int64_t ldx,
                                    const bola_mixed_opts *opts, bola_mixed_info *out, bola_stream_t stream) {
  Workspace *w = reinterpret_cast<Workspace *>(ctx);
  if (!w) return -1;
  return dgesv_mixed_ws(*w, false, n, nrhs, a, lda, b, ldb, x, ldx, opts, out, (cudaStream_t)stream);
}

namespace bola {
namespace {

int dgesv_mixed_ws(Workspace &w, bool chol, int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *b,
                   int64_t ldb, double *x, int64_t ldx, const bola_mixed_opts *opts, bola_mixed_info *out,
                   cudaStream_t s) {
  if (n < 0) return -1;
  if (nrhs < 0 || nrhs > MAXRHS) return -2;
  if (lda < imax(1, n)) return -4;
  if (ldb < imax(1, n)) return -6;
  if (ldx < imax(1, n)) return -8;
  bola_mixed_opts o = {2, 30, 1e-14, 1, 1, 1};
  if (opts) o = *opts;
  if (o.factor_kind < 0 || o.factor_kind > 3) return -9;
  bola_mixed_info info_out;
  std::memset(&info_out, 0, sizeof info_out);
  if (n == 0 || nrhs == 0) {
    if (out) *out = info_out;
    return 0;
  }
  if (n > 8192) return fail(BOLA_ERR_UNSUPPORTED, "bola_dgesv_mixed: n = %lld > 8192", (long long)n);
  BOLA_TRY(ws_reserve(w, n, nrhs, o.factor_kind, s));
  w.fkind = o.factor_kind;
  w.chol = chol;
  const bool fp64 = o.factor_kind == 3;
  const int64_t ldW = fp64 ? cdiv(n, 32) * 32 : n;
  w.ldW = ldW;
  const int nr = (int)nrhs;
  double *nrm = w.norms;  // [0..nr): ||r||, [nr..2nr): ||x||, [2nr..3nr): ||b||, [3nr]: ||A||

  // scale, convert, factor
  if (chol) {
    // W = D A D (lower triangle), D a power of two per row making the diagonal O(1)
    ProfScope prof(s, "mixed_convert", 0.0, 6.0 * (double)n * n, 2);
    sym_scale<<<(unsigned)cdiv(n, 256), 256, 0, s>>>(n, a, lda, w.dscale);
    if (fp64)
      convert_sym_lower<double><<<(unsigned)cdiv(n * n, 256), 256, 0, s>>>(n, a, lda, w.dscale, (double *)w.W, ldW);
    else
      convert_sym_lower<float><<<(unsigned)cdiv(n * n, 256), 256, 0, s>>>(n, a, lda, w.dscale, (float *)w.W, n);
  } else {
    ProfScope prof(s, "mixed_convert", 0.0, 12.0 * (double)n * n, 3);
    BOLA_TRY_CUDA(cudaMemsetAsync(w.scale, 0, sizeof(double) * cdiv(n, TB), s));
    colblock_max<<<dim3((unsigned)cdiv(n, TB), (unsigned)imin(16, cdiv(n, 256))), 256, 0, s>>>(
        n, a, lda, reinterpret_cast<unsigned long long *>(w.scale));
    colblock_finish<<<(unsigned)cdiv(cdiv(n, TB), 256), 256, 0, s>>>(cdiv(n, TB), w.scale);
    if (fp64)
      convert_scaled<double><<<(unsigned)cdiv(n * n, 256), 256, 0, s>>>(n, a, lda, w.scale, (double *)w.W, ldW);
    else
      convert_scaled<float><<<(unsigned)cdiv(n * n, 256), 256, 0, s>>>(n, a, lda, w.scale, (float *)w.W, n);
  }
  BOLA_CHECK_LAUNCH();
  // A's digit planes and its row sums (once per call: a solve handed on to
  // another factor within the same call keeps them)
  if (!w.split_kept) BOLA_TRY(w.oz.split(s, a, lda, w.rowsum));
  {
    ProfScope prof(s, "mixed_norms", 0.0, 8.0 * (double)n * nr, 2);
    max_of<<<1, 1024, 0, s>>>(n, w.rowsum, nrm + 3 * nr);
    col_absmax<<<nr, 256, 0, s>>>(n, b, ldb, nrm + 2 * nr);
  }
  BOLA_CHECK_LAUNCH();
  // The spread max|u_ii| / min|u_ii| of the low-precision U is a cheap lower
  // bound on kappa(A).  Above a per-factor-kind limit neither refinement nor
  // GMRES(24)-IR reaches 1e-14, so the FP64 path is taken at once (if
  // allowed).  The limits sit at the geometric midpoints between the largest
  // spread that converged and the smallest that did not, measured on
  // n = 1024 and 4096 systems with geometric spectra and kappa 1e2/1e6/1e10:
  // bf16 55 | 560, tf32 93 | 1.3e4, 3xTF32 3.6e3 | 5.5e5.  A wrong call costs
  // time only: the refinement attempt before the fallback, or an FP64 solve
  // where the mixed one would have done.  The FP64-accurate factor (kind 3)
  // refines anything its pivots leave below ~1e13.  The spread only grows as
  // pivots are added, so the factorisation itself gives up at the first panel
  // that takes it over the limit, with the decision the whole factor would
  // give, or earlier when the spread is on course for 100 times the limit
  // (give_up_now: log-linear extrapolation from a quarter of the columns on).
  const double limit = o.factor_kind == 0 ? 175.0 : o.factor_kind == 1 ? 1100.0 : o.factor_kind == 2 ? 4.5e4 : 1e13;
  const double give_up = (o.fallback_fp64 || o.escalate) ? limit : INFINITY;
  if (chol) {
    // Cholesky (no pivoting), then its LU form L D^-1, D L^T for the solves
    if (fp64) {
      BOLA_TRY(w.lu.factor_chol64(s, (double *)w.W, ldW, w.info, give_up));
      BOLA_TRY(chol_lu_form<double>(s, n, (double *)w.W, ldW, (double *)w.dg));
    } else {
      BOLA_TRY(w.lu.factor_chol(s, (float *)w.W, n, w.info, give_up));
      BOLA_TRY(chol_lu_form<float>(s, n, (float *)w.W, n, (float *)w.dg));
    }
  } else if (fp64) {
    BOLA_TRY(w.lu.factor64(s, (double *)w.W, ldW, w.ipiv, w.info, give_up, n > TB ? w.perm : nullptr));
  } else {
    BOLA_TRY(w.lu.factor(s, (float *)w.W, n, w.ipiv, w.info, give_up, n > TB ? w.perm : nullptr));
  }
  // the row permutation: kept by the LU's swap kernels for n > 64 (there is
  // no swap kernel when the whole matrix is one panel)
  if (chol || n <= TB) {
    ProfScope prof(s, "mixed_perm");
    if (chol)
      iota_perm<<<(unsigned)cdiv(n, 256), 256, 0, s>>>(n, w.perm);
    else
      compose_perm<<<1, 1024, sizeof(int32_t) * n, s>>>(n, w.ipiv, w.perm);
  }
  {
    ProfScope prof(s, "diag_inverses");
    const unsigned nb = (unsigned)cdiv(n, TB);
    if (fp64) {
      diag_block_inverses<double><<<nb, TB, 0, s>>>(n, (const double *)w.W, ldW, (double *)w.Dl, (double *)w.Du);
      diag_extent<double><<<1, 1024, 0, s>>>(n, (const double *)w.W, ldW, w.norms + 5 * MAXRHS);
    } else {
      diag_block_inverses<float><<<nb, TB, 0, s>>>(n, (const float *)w.W, n, (float *)w.Dl, (float *)w.Du);
      BOLA_TRY(couple(s, n, (const float *)w.W, n, (const float *)w.Dl, (const float *)w.Du,
                      const_cast<float *>(w.ts.Cl), const_cast<float *>(w.ts.Cu)));
      diag_extent<float><<<1, 1024, 0, s>>>(n, (const float *)w.W, n, w.norms + 5 * MAXRHS);
    }
  }
  BOLA_CHECK_LAUNCH();
  double ext[2] = {0.0, 0.0};
  BOLA_TRY_CUDA(cudaMemcpyAsync(ext, w.norms + 5 * MAXRHS, sizeof ext, cudaMemcpyDeviceToHost, s));
  int32_t finfo = 0, ferr = 0;
  uint64_t trk[3] = {0, 0, 0};
  BOLA_TRY_CUDA(cudaMemcpyAsync(trk, w.lu.track, sizeof trk, cudaMemcpyDeviceToHost, s));
  BOLA_TRY_CUDA(cudaMemcpyAsync(&finfo, w.info, sizeof finfo, cudaMemcpyDeviceToHost, s));
  BOLA_TRY_CUDA(cudaMemcpyAsync(&ferr, w.lu.err, sizeof ferr, cudaMemcpyDeviceToHost, s));
  BOLA_TRY_CUDA(cudaStreamSynchronize(s));
  info_out.factor_info = finfo;
  info_out.factorization = chol ? 1 : 0;
  // a bounded wait gave up: 5 the panel's candidate exchange, others a
  // tensor-core update's pipeline (the factor is then unusable)
  if (ferr != 0) return fail(BOLA_ERR_CUDA, "mixed LU: a bounded wait expired (code %d)", ferr);
  if (chol && finfo != 0 && !(o.escalate && o.factor_kind < 3)) {
    // a pivot that is not positive: A is not SPD at this precision (or at
    // all) and no FP64-accurate Cholesky is left to try; the mixed LU takes
    // over with the same options
    w.split_kept = true;
    const int st = dgesv_mixed_ws(w, false, n, nrhs, a, lda, b, ldb, x, ldx, &o, out, s);
    w.split_kept = false;
    BOLA_TRY(st);
    if (out) out->factor_info = finfo;
    return 0;
  }

  bool converged = false;
  double berr = INFINITY, prev = INFINITY;
  int path = 0;
  const bool gave_up = (uint32_t)trk[2] != 0 && !std::isinf(give_up);
  if (gave_up) {  // the extent over the pivots reached (W beyond them is unfinished)
    double mx, mn;
    std::memcpy(&mx, &trk[0], sizeof mx);
    std::memcpy(&mn, &trk[1], sizeof mn);
    ext[0] = mx;
    ext[1] = mn;
  }
  const double spread = ext[1] > 0.0 ? ext[0] / ext[1] : INFINITY;
  info_out.condition_estimate = spread;
  const bool hopeless = gave_up || ((o.fallback_fp64 || o.escalate) && !(spread < limit));
  if (finfo == 0 && !hopeless) {
    // x0 = correction of b (rscale = ||b||)
    BOLA_TRY(correction(s, w, n, nr, b, ldb, nrm + 2 * nr, x, ldx, true));
    bool to_gmres = false;
    for (int it = 0; it <= o.max_iterations; ++it) {
      BOLA_TRY(residual_berr(s, w, n, nr, a, lda, b, ldb, x, ldx, &berr));
      info_out.iterations = it;
      if (berr <= o.tolerance) {
        converged = true;
        break;
      }
      if (it > 0) {
        const double rate = berr / prev;
        if (!(rate < 0.5)) {  // stalled or diverging
          to_gmres = o.gmres != 0;
          break;
        }
        // converging slowly: Krylov acceleration pays.  A plain sweep and a
        // GMRES step cost about the same (two triangular solves and an
        // FP64-accurate product); GMRES(24) took ~13 of them for the seven
        // digits left at kappa = 1e6 (n = 8192), i.e. ~1.9 per digit, and a
        // plain sweep at rate r gains log10(1 / r) digits: the break-even is
        // r ~ 0.3 (kappa = 1e6: r ~ 0.2, plain IR 28.7 against 30.6 ms)
        if (o.gmres && rate > 0.3) {
          to_gmres = true;
          break;
        }
      }
      prev = berr;
      BOLA_TRY(correction(s, w, n, nr, w.r, n, nrm, x, ldx, false));
    }
    if (!converged && to_gmres) {
      // a stalled sweep may have made x worse than the previous one; GMRES-IR
      // starts from the current x and its residual (w.r)
      path = 1;
      double gprev = berr;
      for (int outer = 0; outer < 10; ++outer) {
        BOLA_TRY(gmres_step(s, w, n, nr, a, lda, x, ldx, 1e-8, &info_out.gmres_iterations));
        BOLA_TRY(residual_berr(s, w, n, nr, a, lda, b, ldb, x, ldx, &berr));
        info_out.iterations += 1;
        if (berr <= o.tolerance) {
          converged = true;
          break;
        }
        if (!(berr < 0.5 * gprev)) break;
        gprev = berr;
      }
    }
  }
  info_out.backward_error = berr;
  info_out.path = path;
  if (!converged && o.escalate && o.factor_kind < 3) {
    // the FP64-accurate factor: its own refinement, and its own FP64 fallback
    bola_mixed_opts o3 = o;
    o3.factor_kind = 3;
    o3.escalate = 0;
    bola_mixed_info i3;
    w.split_kept = true;
    const int st = dgesv_mixed_ws(w, chol, n, nrhs, a, lda, b, ldb, x, ldx, &o3, &i3, s);
    w.split_kept = false;
    BOLA_TRY(st);
    i3.iterations += info_out.iterations;
    i3.gmres_iterations += info_out.gmres_iterations;
    if (i3.path != 2) i3.path = 3;
    if (out) *out = i3;
    return 0;
  }
  if (!converged && o.fallback_fp64) {
    // plain FP64 path on a copy of A (BOLA's getrf + laswp + trsm)
    double *acopy = nullptr;
    BOLA_TRY_CUDA(cudaMallocAsync(&acopy, sizeof(double) * n * n, s));
    {
      ProfScope prof(s, "mixed_fallback_copy", 0.0, 16.0 * (double)n * n);
      BOLA_TRY_CUDA(cudaMemcpy2DAsync(acopy, sizeof(double) * n, a, sizeof(double) * lda, sizeof(double) * n, n,
                                      cudaMemcpyDeviceToDevice, s));
      copy_cols<<<(unsigned)cdiv(n * nr, 256), 256, 0, s>>>(n, nr, b, ldb, x, ldx);
    }
    int st = bola_dgetrf(n, n, acopy, n, w.ipiv, w.info, (bola_stream_t)s);
    if (st == 0) st = bola_dgetrs(n, nr, acopy, n, w.ipiv, x, ldx, (bola_stream_t)s);
    cudaFreeAsync(acopy, s);
    if (st != 0) return st;
    info_out.path = 2;
    info_out.factorization = 0;
    // backward error of the FP64 answer
    BOLA_TRY(residual_berr(s, w, n, nr, a, lda, b, ldb, x, ldx, &berr));
    info_out.backward_error = berr;
  }
  if (out) *out = info_out;
  return 0;
}

}  // namespace
}  // namespace bola
