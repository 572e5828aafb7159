// common.cuh — shared helpers of the FP64 path.
//
// Every kernel here reproduces BOLA's IEEE operation sequence, so these
// translation units are compiled with -fmad=false: a product followed by a sum
// is never contracted behind our back.  The only fused multiply-adds are the
// explicit fused() calls, placed exactly where BOLA uses a vector FMA.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "bola_gb300.h"
#include "profile.cuh"

namespace bola {

// ---- host side ------------------------------------------------------------
int fail(int code, const char *fmt, ...);       // records the message, returns code
int cuda_fail(cudaError_t e, const char *what);  // records the CUDA error text
int lanes();                                     // SIMD width reproduced: 2 or 4
int num_sms();                                   // SMs of the current device

#define BOLA_TRY_CUDA(expr)                                   \
  do {                                                        \
    cudaError_t e_ = (expr);                                  \
    if (e_ != cudaSuccess) return ::bola::cuda_fail(e_, #expr); \
  } while (0)
#define BOLA_CHECK_LAUNCH() BOLA_TRY_CUDA(cudaGetLastError())
#define BOLA_TRY(expr)      \
  do {                      \
    int r_ = (expr);        \
    if (r_ != 0) return r_; \
  } while (0)

inline char upc(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 32) : c; }
__host__ __device__ inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline int64_t imin(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ inline int64_t imax(int64_t a, int64_t b) { return a > b ? a : b; }

// Stream-ordered temporary device memory (cudaMallocAsync pool).
class Scratch {
 public:
  Scratch() = default;
  Scratch(const Scratch &) = delete;
  Scratch &operator=(const Scratch &) = delete;
  ~Scratch() { release(); }
  int alloc(size_t bytes, cudaStream_t s) {
    release();
    stream_ = s;
    if (bytes == 0) return 0;
    cudaError_t e = cudaMallocAsync(&ptr_, bytes, s);
    if (e != cudaSuccess) {
      ptr_ = nullptr;
      return cuda_fail(e, "cudaMallocAsync(scratch)");
    }
    return 0;
  }
  void release() {
    if (ptr_) cudaFreeAsync(ptr_, stream_);
    ptr_ = nullptr;
  }
  template <class T>
  T *as() const { return static_cast<T *>(ptr_); }

 private:
  void *ptr_ = nullptr;
  cudaStream_t stream_ = nullptr;
};

// ---- internal launchers shared between translation units -------------------
// Exact DGEMM: per output element, K is walked in chunks of `kc`; each chunk is
// accumulated from zero with fused multiply-adds in increasing k and added to C
// as C = fma(alpha, acc, C) (BOLA's 8x4 micro-kernel, src/gemm.rs:228-336).
// Elements in BOLA's partial 8x4 edge tiles use its unfused scalar kernel
// (src/gemm.rs:357-377).  beta is applied first as BOLA does (src/gemm.rs:110-122).
// tri: 0 = whole C; 1 / 2 = only elements whose 32-block lies strictly above /
// below the block diagonal (the off-diagonal part of a blocked SYRK).
// info: optional device flag; kernels return immediately when *info != 0.
int dgemm_exact(cudaStream_t s, char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
                const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                int64_t ldc, int kc, const int32_t *info, int tri);

int trsm_exact(cudaStream_t s, char side, char uplo, char transa, char diag, int64_t m, int64_t n,
               double alpha, const double *A, int64_t lda, double *B, int64_t ldb,
               const int32_t *info);

int syrk_exact(cudaStream_t s, char uplo, char trans, int64_t n, int64_t k, double alpha,
               const double *A, int64_t lda, double beta, double *C, int64_t ldc,
               const int32_t *info);

int laswp_exact(cudaStream_t s, int64_t n, double *A, int64_t lda, int32_t k1, int32_t k2,
                const int32_t *ipiv, int32_t incx, const int32_t *info);

int getrf2_rec(cudaStream_t s, int64_t m, int64_t n, double *A, int64_t lda, int32_t *ipiv,
               int32_t *info, int32_t col0);

// Look-ahead resources of one blocked factorisation: a high-priority stream
// for the critical path (panels, the next block's columns), a low-priority
// stream for the rest of each trailing update, events, and two device ints.
// Pooled per device, so concurrent callers each take their own set.
struct LookAhead {
  cudaStream_t sp = nullptr, su = nullptr;
  cudaEvent_t ev[8] = {};
  int32_t *snap = nullptr;  // device int32[2]
};
LookAhead *la_acquire();  // nullptr if the resources cannot be created
void la_release(LookAhead *la);

int potrf2_rec(cudaStream_t s, char uplo, int64_t n, double *A, int64_t lda, int32_t *info,
               int32_t col0);

// Adds `add` to ipiv[0..count) unless *info != 0.
int ipiv_add(cudaStream_t s, int32_t *ipiv, int64_t count, int32_t add, const int32_t *info);

// Fused multiply-add of the operands' own precision (templated kernels).
__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }

// Batched small-system solver pieces (batched.cu): the work items of a batch
// (flat int32 records, *nitems of them; group = the 8 per-bucket group sizes
// used) and one persistent launch over items already on the device.
int batch_items(int32_t count, const int32_t *n, const int32_t *kind, const int32_t *group_size,
                std::vector<int32_t> &flat, int32_t *nitems, int *group, double *flops,
                const int32_t *panel_width = nullptr);
int batch_launch(cudaStream_t s, const bola_system *systems, const int32_t *items, int32_t nitems, int32_t *counter,
                 int32_t *info, int tile = 4);

// ---- device side -------------------------------------------------------------
__device__ __forceinline__ double fused(double a, double b, double c) { return __fma_rn(a, b, c); }
// c + t*x with two roundings (BOLA's scalar tails; Rust never contracts).
__device__ __forceinline__ double add_prod(double c, double t, double x) {
  return __dadd_rn(c, __dmul_rn(t, x));
}
__device__ __forceinline__ double sub_prod(double c, double t, double x) {
  return __dsub_rn(c, __dmul_rn(t, x));
}
// Split cluster barrier: ARRIVE (release) and WAIT (acquire), so that work
// between them overlaps the other CTAs' arrival.
__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// x != 0.0 (NaN included) on the integer pipe.  GB300 retires ~2 FP64
// operations per clock per SM and a comparison takes a slot like an FMA, so
// the zero tests inside BOLA's update loops are done on the bits.
__device__ __forceinline__ bool nonzero64(double x) { return (__double_as_longlong(x) << 1) != 0; }
// f ? fma(alpha, x, y) : y + alpha*x (fused body or unfused tail of one of
// BOLA's SIMD loops), with the choice made per warp when the warp agrees: a
// per-lane select would issue the FMA, the multiply and the add for every
// lane (four times the FP64 slots of the FMA alone, measured), while a warp
// whose lanes all take the same form issues only that form.
__device__ __forceinline__ double fused_or_unfused(bool f, double alpha, double x, double y) {
  const unsigned m = __activemask();
  if (__all_sync(m, f)) return __fma_rn(alpha, x, y);
  if (!__any_sync(m, f)) return __dadd_rn(y, __dmul_rn(alpha, x));
  return f ? __fma_rn(alpha, x, y) : __dadd_rn(y, __dmul_rn(alpha, x));
}
__device__ __forceinline__ bool stop_flag(const int32_t *info) {
  return info != nullptr && *(volatile const int32_t *)info != 0;
}

// BOLA's daxpy(len, alpha, x, 1, y, 1) (src/utilities.rs:107-132 / :140-164):
// element idx of the vector body (idx < len rounded down to `lanes`) is fused,
// the scalar tail is not.
// `lanes` is 2 or 4, so rounding down to it is a mask.
__device__ __forceinline__ double daxpy_elem(double y, double alpha, double x, int64_t idx,
                                             int64_t len, int lanes) {
  const int64_t done = len & ~(int64_t)(lanes - 1);
  return fused_or_unfused(idx < done, alpha, x, y);
}

// BOLA's dot_product(n, x, 1, y, 1) (src/utilities.rs:22-54 / :62-92) with
// element strides sx, sy (the unit-stride vector path applied to gathered
// data).  Sequential per lane, then BOLA's horizontal sum and unfused tail.
__device__ __forceinline__ double dot_exact(int64_t n, const double *x, int64_t sx, const double *y,
                                            int64_t sy, int lanes) {
  if (n == 0) return 0.0;
  const int64_t nch = lanes == 4 ? (n >> 2) : (n >> 1);  // n / lanes, lanes 2 or 4
  double l0 = 0.0, l1 = 0.0, l2 = 0.0, l3 = 0.0;
  for (int64_t i = 0; i < nch; ++i) {
    const int64_t b = i * lanes;
    l0 = fused(x[b * sx], y[b * sy], l0);
    l1 = fused(x[(b + 1) * sx], y[(b + 1) * sy], l1);
    if (lanes == 4) {
      l2 = fused(x[(b + 2) * sx], y[(b + 2) * sy], l2);
      l3 = fused(x[(b + 3) * sx], y[(b + 3) * sy], l3);
    }
  }
  double s;
  if (lanes == 4) {
    double h = -0.0;
    h = __dadd_rn(h, l0);
    h = __dadd_rn(h, l1);
    h = __dadd_rn(h, l2);
    h = __dadd_rn(h, l3);
    s = __dadd_rn(0.0, h);
  } else {
    s = __dadd_rn(l0, l1);
  }
  for (int64_t i = nch * lanes; i < n; ++i) s = add_prod(s, x[i * sx], y[i * sy]);
  return s;
}

// Candidate of BOLA's idamax (src/idamax.rs): ordered by value, then by the
// position BOLA's four lane-interleaved accumulators give it.  v = -1 marks
// an element BOLA can never select (NaN; zero in the vector body or tail).
struct Cand {
  int64_t v;  // |x|'s bits (ordered like |x|), or -1 (never selectable) / -2 (no candidate)
  int64_t key;  // smaller wins among equal v
  int64_t idx;  // 0-based index in the searched vector
};
__device__ __forceinline__ bool cand_better(const Cand &a, const Cand &b) {
  return a.v > b.v || (a.v == b.v && a.key < b.key);  // integer compares: no FP64 slots
}
__device__ __forceinline__ Cand make_cand(double x, int64_t idx, int64_t n, int lanes) {
  Cand c;
  c.idx = idx;
  const int64_t ab = __double_as_longlong(x) & INT64_MAX;
  const bool nan = ab > 0x7ff0000000000000LL;
  const int64_t small = lanes == 4 ? 16 : 8;
  if (n < small) {  // scalar path, starts from max = -1.0: any non-NaN qualifies
    c.v = nan ? -1 : ab;
    c.key = idx;
    return c;
  }
  // vector body and tail start from max = 0.0; chunk = 4 * lanes (8 or 16)
  const int sl = lanes == 4 ? 2 : 1, sc = sl + 2;
  const int64_t nch = n >> sc;
  const int64_t nv = nch << sc;
  c.v = (nan || ab == 0) ? -1 : ab;
  if (idx < nv) {
    const int64_t r = idx & ((1 << sc) - 1);
    const int64_t lane = r & (lanes - 1), acc = r >> sl;
    c.key = (lane * 4 + acc) * nch + (idx >> sc);
  } else {
    c.key = idx;
  }
  return c;
}
__device__ __forceinline__ Cand cand_none() {
  Cand c;
  c.v = -2;
  c.key = INT64_MAX;
  c.idx = 0;
  return c;
}
__device__ __forceinline__ Cand shfl_cand(const Cand &c, int src) {
  Cand o;
  o.v = __shfl_sync(0xffffffffu, c.v, src);
  o.key = __shfl_sync(0xffffffffu, c.key, src);
  o.idx = __shfl_sync(0xffffffffu, c.idx, src);
  return o;
}
__device__ __forceinline__ Cand warp_best(Cand c) {
  for (int off = 16; off > 0; off >>= 1) {
    Cand o;
    o.v = __shfl_down_sync(0xffffffffu, c.v, off);
    o.key = __shfl_down_sync(0xffffffffu, c.key, off);
    o.idx = __shfl_down_sync(0xffffffffu, c.idx, off);
    if (cand_better(o, c)) c = o;
  }
  return c;
}

// An ordered list of row interchanges, walked as BOLA's laswp walks ipiv
// (src/laswp.rs:30-37): i from i1 to i2 by i_inc, ipiv index from ix0 by incx.
struct SwapPlan {
  int64_t ix0;
  int32_t i1, i2, i_inc, incx;
};

// Composes the interchanges into "row rows[t] takes the old value of row
// src[t]" (at most 2 entries per interchange; the caller sizes the arrays).
__device__ __forceinline__ int compose_swaps(const SwapPlan &p, const int32_t *ipiv, int64_t *rows,
                                             int64_t *src) {
  int cnt = 0;
  int64_t ix = p.ix0;
  for (int32_t i = p.i1; p.i_inc > 0 ? i <= p.i2 : i >= p.i2; i += p.i_inc, ix += p.incx) {
    const int64_t ip = ipiv[ix];
    if (ip == (int64_t)i) continue;
    const int64_t r1 = (int64_t)i - 1, r2 = ip - 1;
    int a = -1, b = -1;
    for (int t = 0; t < cnt; ++t) {
      if (rows[t] == r1) a = t;
      if (rows[t] == r2) b = t;
    }
    if (a < 0) {
      rows[cnt] = r1;
      src[cnt] = r1;
      a = cnt++;
    }
    if (b < 0) {
      rows[cnt] = r2;
      src[cnt] = r2;
      b = cnt++;
    }
    const int64_t t = src[a];
    src[a] = src[b];
    src[b] = t;
  }
  return cnt;
}

// Warp-cooperative compose_swaps for at most 16*E interchanges (E = 2: the
// 32-column getrf panel; E = 4: the 64-column mixed-precision panel): lanes
// prefetch the pivots, each lane keeps entries lane + 32*e in registers,
// lookups are ballots.  Called by all 32 lanes of one warp; writes rows/src
// (>= 32*E entries) and returns the count on every lane.
template <int E = 2, typename RowT = int64_t>
__device__ __forceinline__ int compose_swaps_warp(const SwapPlan &p, const int32_t *ipiv, RowT *rows, RowT *src) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int nsw = p.i_inc > 0 ? p.i2 - p.i1 + 1 : p.i1 - p.i2 + 1;
  int64_t my_ip[E / 2];
#pragma unroll
  for (int h = 0; h < E / 2; ++h) {
    const int t = lane + 32 * h;
    my_ip[h] = t < nsw ? (int64_t)ipiv[p.ix0 + (int64_t)t * p.incx] : 0;
  }
  int64_t R[E], S[E];
#pragma unroll
  for (int e = 0; e < E; ++e) R[e] = S[e] = -1;
  int cnt = 0;
  for (int t = 0; t < nsw; ++t) {
    const int32_t i = p.i1 + t * p.i_inc;
    int64_t ip = 0;
#pragma unroll
    for (int h = 0; h < E / 2; ++h) {
      const int64_t v = __shfl_sync(FULL, my_ip[h], t & 31);
      if ((t >> 5) == h) ip = v;
    }
    if (ip == (int64_t)i) continue;
    const int64_t want[2] = {(int64_t)i - 1, ip - 1};
    int slot[2];
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      int s = -1;
#pragma unroll
      for (int e = E - 1; e >= 0; --e) {
        const unsigned mk = __ballot_sync(FULL, lane + 32 * e < cnt && R[e] == want[w]);
        if (mk) s = 32 * e + __ffs(mk) - 1;
      }
      if (s < 0) {
        s = cnt++;
#pragma unroll
        for (int e = 0; e < E; ++e)
          if (lane == (s & 31) && (s >> 5) == e) {
            R[e] = want[w];
            S[e] = want[w];
          }
      }
      slot[w] = s;
    }
    int64_t sa = 0, sb = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int64_t va = __shfl_sync(FULL, S[e], slot[0] & 31);
      const int64_t vb = __shfl_sync(FULL, S[e], slot[1] & 31);
      if ((slot[0] >> 5) == e) sa = va;
      if ((slot[1] >> 5) == e) sb = vb;
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if (lane == (slot[0] & 31) && (slot[0] >> 5) == e) S[e] = sb;
      if (lane == (slot[1] & 31) && (slot[1] >> 5) == e) S[e] = sa;
    }
  }
#pragma unroll
  for (int e = 0; e < E; ++e)
    if (lane + 32 * e < cnt) {
      rows[lane + 32 * e] = (RowT)R[e];
      src[lane + 32 * e] = (RowT)S[e];
    }
  return cnt;
}

}  // namespace bola
