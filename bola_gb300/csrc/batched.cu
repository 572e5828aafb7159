// batched.cu — many small independent solves of uneven size in one persistent
// launch (no BOLA counterpart; each system's answer must match BOLA's FP64
// getrf/potrf + trsm solve within rounding).
//
// Plan (host, once per batch shape): systems are bucketed by order n; each
// bucket has a group size G (threads per system: 32, 64, 128 or 256, from the
// autotuned table) and work items of 256/G systems of that bucket, ordered by
// decreasing cost (largest first, for load balance).  Solve (device): a grid
// of persistent 256-thread CTAs pulls items from an atomic counter; the CTA
// splits into 256/G groups, each factoring one system in place in global
// memory (L2-resident: at most 512 KB per system) with partial pivoting (LU)
// or Cholesky in panels of 8 columns (register-tiled trailing updates), and
// then solving its right-hand sides.  A group synchronises
// with its own named barrier, so a system's arithmetic never depends on which
// systems share its CTA: every result is the same alone and in any mix.
// FP64 throughout; all waits are barriers (no spin loops).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace bola {
namespace {

constexpr int BT = 256;         // threads per CTA
constexpr int MAXG = BT / 32;   // groups per CTA at most
constexpr int ITEM = 3 + MAXG;  // ints per work item: G, count, panel width, system ids
constexpr int NBUCKET = 8;
// upper n of each bucket (inclusive)
constexpr int BUCKET_N[NBUCKET] = {16, 32, 48, 64, 96, 128, 192, 1 << 30};

struct SystemDesc {
  int32_t n, nrhs, kind, lda, ldb, pad;
  double *a, *b;
};
static_assert(sizeof(SystemDesc) == sizeof(bola_system), "bola_system layout");

__device__ __forceinline__ void group_sync(int G, int g) {
  if (G == 32) {
    __syncwarp();
  } else if (G == BT) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(G) : "memory");
  }
}

// argmax |A[k:n, k]| within a group; ties -> lowest row; NaN never wins.
// The comparisons run on the integer pipe: |v|'s bits order like |v| (a
// double comparison would take a slot of the narrow FP64 pipe per element).
// red: 2*MAXG scratch per group.
__device__ int group_argmax(const double *col, int k, int n, int t, int G, int g, long long *redv, int *redi) {
  long long best = -1;
  int bi = k;
  for (int i = k + t; i < n; i += G) {
    const long long v = __double_as_longlong(col[i]) & 0x7fffffffffffffffll;
    if (v <= 0x7ff0000000000000ll && v > best) {
      best = v;
      bi = i;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    const long long ov = __shfl_down_sync(0xffffffffu, best, off);
    const int oi = __shfl_down_sync(0xffffffffu, bi, off);
    if (ov > best || (ov == best && oi < bi)) {
      best = ov;
      bi = oi;
    }
  }
  const int w = t >> 5, nw = G >> 5;
  if ((t & 31) == 0) {
    redv[w] = best;
    redi[w] = bi;
  }
  group_sync(G, g);
  long long b = redv[0];
  int r = redi[0];
  for (int q = 1; q < nw; ++q)
    if (redv[q] > b || (redv[q] == b && redi[q] < r)) {
      b = redv[q];
      r = redi[q];
    }
  group_sync(G, g);
  return r;
}

// ---- blocked factorisation pieces -------------------------------------------
// The factorisations below run in panels of PB columns: pivots inside the
// panel update only the panel's columns; the rest of the matrix then gets the
// whole panel at once (U12 by a small forward substitution, A22 by register
// tiles of TR x TC elements per thread), so each trailing element is loaded
// and stored once per panel instead of once per pivot.  Every element still
// receives fma(-l_ik, u_kj, a_ij) for k in increasing order, with the values
// the unblocked order gives it (row interchanges move whole rows, deferred
// updates included), so results are those of the unblocked algorithm, bit for
// bit.
// The panel width PB (8, 12 or 16 columns) is chosen per size bucket and
// travels with each work item; the register tile TR x TC (TC = 4, TR = 4 or
// 2) is chosen per plan, since it sets the kernel's register count.  Neither
// changes any element's sequence of operations.
constexpr int TC = 4;

// A[c0:n, c0:n] -= A[c0:n, k0:k0+kb] * A[k0:k0+kb, c0:n] (lower = false), or
// its lower triangle -= A[c0:n, k0:k0+kb] * A[c0:n, k0:k0+kb]^T (lower = true),
// with c0 = k0 + kb.
template <int TR>
__device__ void group_trailing(double *A, int lda, int n, int k0, int kb, bool lower, int t, int G) {
  const int c0 = k0 + kb, m2 = n - c0;
  if (m2 <= 0) return;
  const int tr = (m2 + TR - 1) / TR, tc = (m2 + TC - 1) / TC;
  // tile (ti, tj): the full tr x tc grid, or its lower triangle (ti >= tj) packed by columns
  int ti = t, tj = 0, dq = 0, dr = 0;
  if (lower) {
    while (ti >= tr && tj < tr) {
      ti -= tr - tj - 1;
      ++tj;
    }
  } else {
    dq = G / tr;
    dr = G % tr;
    ti = t % tr;
    tj = t / tr;
  }
  const int ntiles = lower ? tr * (tr + 1) / 2 : tr * tc;
  for (int e = t; e < ntiles; e += G) {
    const int i0 = c0 + ti * TR, j0 = c0 + tj * TC;
    double acc[TR][TC];
#pragma unroll
    for (int r = 0; r < TR; ++r)
#pragma unroll
      for (int c = 0; c < TC; ++c) {
        const int i = i0 + r, j = j0 + c;
        acc[r][c] = (i < n && j < n) ? A[i + (int64_t)j * lda] : 0.0;
      }
    for (int q = 0; q < kb; ++q) {
      const int64_t kq = (int64_t)(k0 + q) * lda;
      double l[TR], u[TC];
#pragma unroll
      for (int r = 0; r < TR; ++r) l[r] = i0 + r < n ? A[i0 + r + kq] : 0.0;
#pragma unroll
      for (int c = 0; c < TC; ++c)
        u[c] = j0 + c < n ? (lower ? A[j0 + c + kq] : A[(k0 + q) + (int64_t)(j0 + c) * lda]) : 0.0;
#pragma unroll
      for (int r = 0; r < TR; ++r)
#pragma unroll
        for (int c = 0; c < TC; ++c) acc[r][c] = fma(-l[r], u[c], acc[r][c]);
    }
#pragma unroll
    for (int r = 0; r < TR; ++r)
#pragma unroll
      for (int c = 0; c < TC; ++c) {
        const int i = i0 + r, j = j0 + c;
        if (i < n && j < n && (!lower || i >= j)) A[i + (int64_t)j * lda] = acc[r][c];
      }
    if (lower) {
      ti += G;
      while (ti >= tr && tj < tr) {
        ti -= tr - tj - 1;
        ++tj;
      }
    } else {
      ti += dr;
      tj += dq;
      if (ti >= tr) {
        ti -= tr;
        ++tj;
      }
    }
  }
}

// U12 = L11^-1 A12 for the panel rows k0..k0+kb-1 (unit lower L11), a column
// per thread: row r takes fma(-l_rq, u_q, u_r) for q < r in increasing q.
template <int PB>
__device__ void group_u12(double *A, int lda, int n, int k0, int kb, int t, int G) {
  for (int j = k0 + kb + t; j < n; j += G) {
    double u[PB];
#pragma unroll
    for (int r = 0; r < PB; ++r) u[r] = r < kb ? A[(k0 + r) + (int64_t)j * lda] : 0.0;
#pragma unroll
    for (int q = 0; q < PB - 1; ++q)
#pragma unroll
      for (int r = q + 1; r < PB; ++r)
        if (r < kb) u[r] = fma(-A[(k0 + r) + (int64_t)(k0 + q) * lda], u[q], u[r]);
#pragma unroll
    for (int r = 1; r < PB; ++r)
      if (r < kb) A[(k0 + r) + (int64_t)j * lda] = u[r];
  }
}

// LU with partial pivoting of one system by a group; the row interchanges are
// applied to B as they happen, then L y = P b and U x = y.
template <int PB, int TR>
__device__ int group_lu_solve(const SystemDesc &S, int t, int G, int g, long long *redv, int *redi, double *sinv) {
  const int n = S.n, lda = S.lda, ldb = S.ldb, nr = S.nrhs;
  double *A = S.a, *B = S.b;
  int info = 0;
  for (int k = 0; k < n; ++k) {
    const int p = group_argmax(A + (int64_t)k * lda, k, n, t, G, g, redv, redi);
    const double piv = A[p + (int64_t)k * lda];
    if (!nonzero64(piv)) {
      info = k + 1;
      break;
    }
    if (t == 0) *sinv = 1.0 / piv;  // once per group; published by the barrier below
    if (p != k) {
      for (int j = t; j < n; j += G) {
        const double tmp = A[k + (int64_t)j * lda];
        A[k + (int64_t)j * lda] = A[p + (int64_t)j * lda];
        A[p + (int64_t)j * lda] = tmp;
      }
      for (int c = t; c < nr; c += G) {
        const double tmp = B[k + (int64_t)c * ldb];
        B[k + (int64_t)c * ldb] = B[p + (int64_t)c * ldb];
        B[p + (int64_t)c * ldb] = tmp;
      }
    }
    group_sync(G, g);
    const double inv = *sinv;
    for (int i = k + 1 + t; i < n; i += G) A[i + (int64_t)k * lda] *= inv;
    group_sync(G, g);
    // the rank-1 update on the rest of this panel's columns; the columns after
    // the panel get the whole panel at once below
    const int k0 = k - k % PB, kend = k0 + PB < n ? k0 + PB : n;
    const int m = n - k - 1, w = kend - k - 1;
    if (m > 0 && w > 0) {
      // element e = t, t + G, ... of the m x w block, (i, j) advanced without a
      // division per element
      const int dq = G / m, dr = G % m;
      int i = k + 1 + t % m, j = k + 1 + t / m;
      for (int e = t; e < m * w; e += G) {
        A[i + (int64_t)j * lda] = fma(-A[i + (int64_t)k * lda], A[k + (int64_t)j * lda], A[i + (int64_t)j * lda]);
        i += dr;
        j += dq;
        if (i >= n) {
          i -= m;
          ++j;
        }
      }
    }
    group_sync(G, g);
    if (k + 1 == kend && kend < n) {  // the panel is done: U12, then A22
      group_u12<PB>(A, lda, n, k0, kend - k0, t, G);
      group_sync(G, g);
      group_trailing<TR>(A, lda, n, k0, kend - k0, false, t, G);
      group_sync(G, g);
    }
  }
  if (info) return info;
  // forward: unit lower
  for (int k = 0; k < n; ++k) {
    const int m = n - k - 1;
    if (m > 0) {
      const int dq = G / m, dr = G % m;
      int i = k + 1 + t % m, c = t / m;
      for (int e = t; e < m * nr; e += G) {
        B[i + (int64_t)c * ldb] = fma(-A[i + (int64_t)k * lda], B[k + (int64_t)c * ldb], B[i + (int64_t)c * ldb]);
        i += dr;
        c += dq;
        if (i >= n) {
          i -= m;
          ++c;
        }
      }
    }
    group_sync(G, g);
  }
  // backward: upper
  for (int k = n - 1; k >= 0; --k) {
    for (int c = t; c < nr; c += G) B[k + (int64_t)c * ldb] /= A[k + (int64_t)k * lda];
    group_sync(G, g);
    if (k > 0) {
      const int dq = G / k, dr = G % k;
      int i = t % k, c = t / k;
      for (int e = t; e < k * nr; e += G) {
        B[i + (int64_t)c * ldb] = fma(-A[i + (int64_t)k * lda], B[k + (int64_t)c * ldb], B[i + (int64_t)c * ldb]);
        i += dr;
        c += dq;
        if (i >= k) {
          i -= k;
          ++c;
        }
      }
    }
    group_sync(G, g);
  }
  return 0;
}

// Cholesky A = L L^T (lower) of one system by a group, then L y = b, L^T x = y.
template <int PB, int TR>
__device__ int group_chol_solve(const SystemDesc &S, int t, int G, int g, double *sinv) {
  const int n = S.n, lda = S.lda, ldb = S.ldb, nr = S.nrhs;
  double *A = S.a, *B = S.b;
  for (int k = 0; k < n; ++k) {
    const double d = A[k + (int64_t)k * lda];
    // d > 0 (NaN excluded) on the bits
    const long long db = __double_as_longlong(d);
    if (!(db > 0 && db <= 0x7ff0000000000000ll)) return k + 1;
    // the square root and its reciprocal once per group, not once per thread
    double r = 0.0;
    if (t == 0) {
      r = sqrt(d);
      *sinv = 1.0 / r;
    }
    group_sync(G, g);
    if (t == 0) A[k + (int64_t)k * lda] = r;
    const double inv = *sinv;
    for (int i = k + 1 + t; i < n; i += G) A[i + (int64_t)k * lda] *= inv;
    group_sync(G, g);
    // the rank-1 update on the rest of this panel's columns, lower part only,
    // packed column by column (column jj, global k+1+jj, holds rows jj..m-1):
    // walking the full square would issue the FP64 update for the upper half
    // too, predicated off
    const int k0 = k - k % PB, kend = k0 + PB < n ? k0 + PB : n;
    const int m = n - k - 1, w = kend - k - 1;
    if (m > 0 && w > 0) {
      int ii = t, jj = 0;
      while (ii >= m && jj < w) {
        ii -= m - jj - 1;
        ++jj;
      }
      const int total = w * m - w * (w - 1) / 2;
      for (int e = t; e < total; e += G) {
        const int i = k + 1 + ii, j = k + 1 + jj;
        A[i + (int64_t)j * lda] = fma(-A[i + (int64_t)k * lda], A[j + (int64_t)k * lda], A[i + (int64_t)j * lda]);
        ii += G;
        while (ii >= m && jj < w) {
          ii -= m - jj - 1;
          ++jj;
        }
      }
    }
    group_sync(G, g);
    if (k + 1 == kend && kend < n) {  // the panel is done: the trailing lower triangle
      group_trailing<TR>(A, lda, n, k0, kend - k0, true, t, G);
      group_sync(G, g);
    }
  }
  for (int k = 0; k < n; ++k) {  // L y = b
    for (int c = t; c < nr; c += G) B[k + (int64_t)c * ldb] /= A[k + (int64_t)k * lda];
    group_sync(G, g);
    const int m = n - k - 1;
    if (m > 0) {
      const int dq = G / m, dr = G % m;
      int i = k + 1 + t % m, c = t / m;
      for (int e = t; e < m * nr; e += G) {
        B[i + (int64_t)c * ldb] = fma(-A[i + (int64_t)k * lda], B[k + (int64_t)c * ldb], B[i + (int64_t)c * ldb]);
        i += dr;
        c += dq;
        if (i >= n) {
          i -= m;
          ++c;
        }
      }
    }
    group_sync(G, g);
  }
  for (int k = n - 1; k >= 0; --k) {  // L^T x = y
    for (int c = t; c < nr; c += G) B[k + (int64_t)c * ldb] /= A[k + (int64_t)k * lda];
    group_sync(G, g);
    if (k > 0) {
      const int dq = G / k, dr = G % k;
      int i = t % k, c = t / k;
      for (int e = t; e < k * nr; e += G) {
        B[i + (int64_t)c * ldb] = fma(-A[k + (int64_t)i * lda], B[k + (int64_t)c * ldb], B[i + (int64_t)c * ldb]);
        i += dr;
        c += dq;
        if (i >= k) {
          i -= k;
          ++c;
        }
      }
    }
    group_sync(G, g);
  }
  return 0;
}

template <int PB, int TR>
__device__ int group_solve(const SystemDesc &S, int t, int G, int g, long long *redv, int *redi, double *sinv) {
  return S.kind == 1 ? group_chol_solve<PB, TR>(S, t, G, g, sinv) : group_lu_solve<PB, TR>(S, t, G, g, redv, redi, sinv);
}

template <int TR>
__global__ void __launch_bounds__(BT)
batched_solve_kernel(const SystemDesc *__restrict__ sys, const int32_t *__restrict__ items, int32_t nitems,
                     int32_t *counter, int32_t *info) {
  __shared__ int32_t cur[ITEM];
  __shared__ long long redv[MAXG][MAXG];
  __shared__ double sinv[MAXG];
  __shared__ int redi[MAXG][MAXG];
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) {
      const int it = atomicAdd(counter, 1);
      cur[0] = it < nitems ? items[(int64_t)it * ITEM] : 0;
      for (int q = 1; q < ITEM; ++q) cur[q] = it < nitems ? items[(int64_t)it * ITEM + q] : 0;
    }
    __syncthreads();
    const int G = cur[0];
    if (G == 0) break;
    const int g = tid / G, t = tid % G;
    if (g < cur[1]) {
      const int id = cur[3 + g];
      const SystemDesc S = sys[id];
      const int pb = cur[2];
      const int r = pb == 16   ? group_solve<16, TR>(S, t, G, g, redv[g], redi[g], &sinv[g])
                    : pb == 12 ? group_solve<12, TR>(S, t, G, g, redv[g], redi[g], &sinv[g])
                               : group_solve<8, TR>(S, t, G, g, redv[g], redi[g], &sinv[g]);
      if (t == 0) info[id] = r;
    }
    __syncthreads();
  }
}

struct Plan {
  int32_t count = 0, nitems = 0;
  int32_t *items = nullptr;    // device
  int32_t *counter = nullptr;  // device
  int grid = 0;
  double flops = 0.0;
  int group[NBUCKET];
  int tile = 4;  // register tile rows of the kernel (4 or 2)
  cudaGraphExec_t exec = nullptr;
  const void *g_sys = nullptr;
  const void *g_info = nullptr;
};

int bucket_of(int n) {
  int b = 0;
  while (n > BUCKET_N[b]) ++b;
  return b;
}

}  // namespace

// Work items of a batch: per size bucket, systems by decreasing n, BT/G
// systems per item; items by decreasing cost.  flat holds ITEM int32 per item.
int batch_items(int32_t count, const int32_t *n, const int32_t *kind, const int32_t *group_size,
                std::vector<int32_t> &flat, int32_t *nitems, int *group, double *flops, const int32_t *panel_width) {
  static const int kDefault[NBUCKET] = {32, 32, 64, 64, 128, 128, 256, 256};
  int pbw[NBUCKET];
  for (int b = 0; b < NBUCKET; ++b) {
    int gsz = group_size ? group_size[b] : kDefault[b];
    if (gsz != 32 && gsz != 64 && gsz != 128 && gsz != 256) gsz = kDefault[b];
    group[b] = gsz;
    const int pw = panel_width ? panel_width[b] : 8;
    pbw[b] = (pw == 12 || pw == 16) ? pw : 8;
  }
  double fl = 0.0;
  std::vector<std::vector<int>> byb(NBUCKET);
  for (int i = 0; i < count; ++i) {
    if (n[i] < 1 || n[i] > 256)
      return fail(-2, "bola_batch_plan_create: system %d has n = %d (supported 1..256)", i, n[i]);
    byb[bucket_of(n[i])].push_back(i);
    const double nn = n[i];
    fl += (kind && kind[i] == 1) ? nn * nn * nn / 3.0 : 2.0 * nn * nn * nn / 3.0;
  }
  struct It {
    double cost;
    std::vector<int32_t> v;
  };
  std::vector<It> its;
  for (int b = 0; b < NBUCKET; ++b) {
    auto &ids = byb[b];
    std::sort(ids.begin(), ids.end(), [&](int x, int y) { return n[x] > n[y] || (n[x] == n[y] && x < y); });
    const int G = group[b], per = BT / G;
    for (size_t s = 0; s < ids.size(); s += per) {
      It it;
      it.v.assign(ITEM, 0);
      it.v[0] = G;
      it.v[2] = pbw[b];
      int c = 0;
      double cost = 0.0;
      for (size_t q = s; q < ids.size() && c < per; ++q, ++c) {
        it.v[3 + c] = ids[q];
        cost = std::max(cost, (double)n[ids[q]] * n[ids[q]] * n[ids[q]] / G);
      }
      it.v[1] = c;
      it.cost = cost;
      its.push_back(std::move(it));
    }
  }
  std::stable_sort(its.begin(), its.end(), [](const It &x, const It &y) { return x.cost > y.cost; });
  flat.assign(its.size() * ITEM, 0);
  for (size_t i = 0; i < its.size(); ++i) std::memcpy(&flat[i * ITEM], its[i].v.data(), sizeof(int32_t) * ITEM);
  if (flops) *flops = fl;
  if (nitems) *nitems = (int32_t)its.size();
  return 0;
}

int batch_grid(int32_t nitems, int tile) {
  int occ = 0;
  if (tile == 2)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched_solve_kernel<2>, BT, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched_solve_kernel<4>, BT, 0);
  return std::max(1, std::min((int)nitems, num_sms() * std::max(occ, 1)));
}

void launch_kernel(cudaStream_t s, int tile, int grid, const bola_system *systems, const int32_t *items,
                   int32_t nitems, int32_t *counter, int32_t *info) {
  const SystemDesc *sd = reinterpret_cast<const SystemDesc *>(systems);
  if (tile == 2)
    batched_solve_kernel<2><<<grid, BT, 0, s>>>(sd, items, nitems, counter, info);
  else
    batched_solve_kernel<4><<<grid, BT, 0, s>>>(sd, items, nitems, counter, info);
}

// One persistent launch over nitems work items (device array); *counter is
// the work queue's head and is reset here.
int batch_launch(cudaStream_t s, const bola_system *systems, const int32_t *items, int32_t nitems, int32_t *counter,
                 int32_t *info, int tile) {
  if (nitems == 0) return 0;
  BOLA_TRY_CUDA(cudaMemsetAsync(counter, 0, sizeof(int32_t), s));
  launch_kernel(s, tile, batch_grid(nitems, tile), systems, items, nitems, counter, info);
  BOLA_CHECK_LAUNCH();
  return 0;
}

namespace {

}  // namespace
}  // namespace bola

using namespace bola;

extern "C" {

int bola_batch_plan_create_tuned(int32_t count, const int32_t *n, const int32_t *kind,
                                 const bola_batch_tuning *tuning, bola_batch_plan *plan_out) {
  if (count < 0) return -1;
  if (!plan_out) return -5;
  if (tuning && tuning->tile_rows != 0 && tuning->tile_rows != 2 && tuning->tile_rows != 4) return -4;
  Plan *P = new Plan();
  P->count = count;
  P->tile = (tuning && tuning->tile_rows == 2) ? 2 : 4;
  std::vector<int32_t> flat;
  const int st = batch_items(count, n, kind, tuning ? tuning->group_size : nullptr, flat, &P->nitems, P->group,
                             &P->flops, tuning ? tuning->panel_width : nullptr);
  if (st != 0) {
    delete P;
    return st;
  }
  if (cudaMalloc(&P->items, sizeof(int32_t) * std::max<size_t>(flat.size(), 1)) != cudaSuccess ||
      cudaMalloc(&P->counter, sizeof(int32_t)) != cudaSuccess) {
    delete P;
    return fail(BOLA_ERR_CUDA, "bola_batch_plan_create: device allocation failed");
  }
  if (!flat.empty()) cudaMemcpy(P->items, flat.data(), sizeof(int32_t) * flat.size(), cudaMemcpyHostToDevice);
  P->grid = batch_grid(P->nitems, P->tile);
  *plan_out = reinterpret_cast<bola_batch_plan>(P);
  return 0;
}

int bola_batch_plan_create(int32_t count, const int32_t *n, const int32_t *kind, const int32_t *group_size,
                           bola_batch_plan *plan_out) {
  bola_batch_tuning t;
  std::memset(&t, 0, sizeof t);
  if (group_size) std::memcpy(t.group_size, group_size, sizeof t.group_size);
  return bola_batch_plan_create_tuned(count, n, kind, &t, plan_out);
}

int bola_batch_solve(bola_batch_plan plan, const bola_system *systems, int32_t *info, bola_stream_t stream) {
  Plan *P = reinterpret_cast<Plan *>(plan);
  if (!P) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  if (P->nitems == 0) return 0;
  ProfScope prof(s, "batched_solve", P->flops, 0.0, 2);
  BOLA_TRY_CUDA(cudaMemsetAsync(P->counter, 0, sizeof(int32_t), s));
  launch_kernel(s, P->tile, P->grid, systems, P->items, P->nitems, P->counter, info);
  BOLA_CHECK_LAUNCH();
  return 0;
}

int bola_batch_solve_graph(bola_batch_plan plan, const bola_system *systems, int32_t *info, bola_stream_t stream) {
  Plan *P = reinterpret_cast<Plan *>(plan);
  if (!P) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  if (P->nitems == 0) return 0;
  if (P->exec && (P->g_sys != systems || P->g_info != info)) {
    cudaGraphExecDestroy(P->exec);
    P->exec = nullptr;
  }
  if (!P->exec) {
    cudaStream_t cap;
    BOLA_TRY_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g;
    BOLA_TRY_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(P->counter, 0, sizeof(int32_t), cap);
    launch_kernel(cap, P->tile, P->grid, systems, P->items, P->nitems, P->counter, info);
    BOLA_TRY_CUDA(cudaStreamEndCapture(cap, &g));
    BOLA_TRY_CUDA(cudaGraphInstantiate(&P->exec, g, 0));
    cudaGraphDestroy(g);
    cudaStreamDestroy(cap);
    P->g_sys = systems;
    P->g_info = info;
  }
  ProfScope prof(s, "batched_solve", P->flops, 0.0, 2);
  BOLA_TRY_CUDA(cudaGraphLaunch(P->exec, s));
  return 0;
}

int bola_batch_plan_info(bola_batch_plan plan, int32_t *nitems, int32_t *grid, double *flops) {
  Plan *P = reinterpret_cast<Plan *>(plan);
  if (!P) return -1;
  if (nitems) *nitems = P->nitems;
  if (grid) *grid = P->grid;
  if (flops) *flops = P->flops;
  return 0;
}

int bola_batch_plan_destroy(bola_batch_plan plan) {
  Plan *P = reinterpret_cast<Plan *>(plan);
  if (!P) return 0;
  if (P->exec) cudaGraphExecDestroy(P->exec);
  if (P->items) cudaFree(P->items);
  if (P->counter) cudaFree(P->counter);
  delete P;
  return 0;
}

}  // extern "C"

// ---- the tuning table on disk --------------------------------------------------
namespace {

// The integers of the JSON array that follows "key": in text (at most cap).
int json_ints(const std::string &text, const char *key, int32_t *out, int cap) {
  const std::string k = std::string("\"") + key + "\"";
  size_t p = text.find(k);
  if (p == std::string::npos) return -1;
  p = text.find_first_not_of(" \t\r\n:", p + k.size());
  if (p == std::string::npos) return -1;
  if (text[p] != '[') {  // a scalar
    char *end = nullptr;
    const long v = std::strtol(text.c_str() + p, &end, 10);
    if (end == text.c_str() + p) return -1;
    out[0] = (int32_t)v;
    return 1;
  }
  int cnt = 0;
  ++p;
  while (cnt < cap) {
    p = text.find_first_not_of(" \t\r\n,", p);
    if (p == std::string::npos) return -1;
    if (text[p] == ']') break;
    char *end = nullptr;
    const long v = std::strtol(text.c_str() + p, &end, 10);
    if (end == text.c_str() + p) return -1;
    out[cnt++] = (int32_t)v;
    p = (size_t)(end - text.c_str());
  }
  return cnt;
}

}  // namespace

extern "C" int bola_batch_tuning_save(const char *path, const bola_batch_tuning *t) {
  if (!path || !t) return -1;
  FILE *f = std::fopen(path, "w");
  if (!f) return fail(-2, "bola_batch_tuning_save: cannot write %s", path);
  int dev = 0;
  cudaDeviceProp prop;
  std::memset(&prop, 0, sizeof prop);
  if (cudaGetDevice(&dev) == cudaSuccess) cudaGetDeviceProperties(&prop, dev);
  std::fprintf(f, "{\n  \"format\": \"bola_gb300 batched tuning 1\",\n  \"device\": \"%s\",\n  \"sms\": %d,\n",
               prop.name, prop.multiProcessorCount);
  const int32_t *arrs[2] = {t->group_size, t->panel_width};
  const char *names[2] = {"group_size", "panel_width"};
  for (int a = 0; a < 2; ++a) {
    std::fprintf(f, "  \"%s\": [", names[a]);
    for (int b = 0; b < NBUCKET; ++b) std::fprintf(f, "%d%s", arrs[a][b], b + 1 < NBUCKET ? ", " : "");
    std::fprintf(f, "],\n");
  }
  std::fprintf(f, "  \"tile_rows\": %d\n}\n", t->tile_rows);
  std::fclose(f);
  return 0;
}

extern "C" int bola_batch_tuning_load(const char *path, bola_batch_tuning *t, int32_t *sms_recorded) {
  if (!path || !t) return -1;
  FILE *f = std::fopen(path, "r");
  if (!f) return fail(-2, "bola_batch_tuning_load: cannot read %s", path);
  std::string text;
  char buf[4096];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
  std::fclose(f);
  bola_batch_tuning r;
  std::memset(&r, 0, sizeof r);
  int32_t sms = 0;
  if (json_ints(text, "group_size", r.group_size, NBUCKET) != NBUCKET ||
      json_ints(text, "panel_width", r.panel_width, NBUCKET) != NBUCKET ||
      json_ints(text, "tile_rows", &r.tile_rows, 1) != 1)
    return fail(-2, "bola_batch_tuning_load: %s is not a tuning table", path);
  json_ints(text, "sms", &sms, 1);
  for (int b = 0; b < NBUCKET; ++b) {
    const int g = r.group_size[b], w = r.panel_width[b];
    if ((g != 0 && g != 32 && g != 64 && g != 128 && g != 256) || (w != 0 && w != 8 && w != 12 && w != 16))
      return fail(-3, "bola_batch_tuning_load: bucket %d has group %d / panel width %d", b, g, w);
  }
  if (r.tile_rows != 0 && r.tile_rows != 2 && r.tile_rows != 4)
    return fail(-3, "bola_batch_tuning_load: tile_rows %d", r.tile_rows);
  *t = r;
  if (sms_recorded) *sms_recorded = sms;
  return 0;
}
