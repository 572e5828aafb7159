// getrf.cu — LU with partial pivoting, BOLA's blocking and rounding
// (src/getrf.rs:37-101, src/getrf2.rs:39-185).
//
// Blocked right-looking LU with BOLA's NB = 32.  Per block column:
//   1. panel_lu_split: one thread-block CLUSTER (up to 16 CTAs, the panel's
//      rows spread over them and held in shared memory) factors the
//      (m-j) x 32 panel column by column: warp-shuffle idamax under BOLA's
//      lane order, candidate rows pushed through distributed shared memory,
//      reciprocal scale and BOLA's pairwise rank-1 update — one split cluster
//      barrier per column (panel_lu, rows in global memory, for taller panels).
//   2. step_swap_trsm: the 32 row interchanges applied to every other column
//      (BOLA's two laswp calls) fused with BOLA's 32-row unit-lower trsm on
//      the right block row.
//   3. the exact DGEMM for the rank-32 trailing update (from n = 512 on split:
//      the next panel's columns on a high-priority stream, the rest overlapping
//      the next panel on a low-priority one).
// Every element sees the same operation sequence as in BOLA, so A and ipiv
// come out bit-identical (for the SIMD width selected).
#include <cooperative_groups.h>

#include <mutex>
#include <vector>

#include "common.cuh"
#include "sm100.cuh"

namespace cg = cooperative_groups;

namespace bola {
namespace {

constexpr int PNB = 32;   // panel width: BOLA's NB (src/getrf.rs:11) / recursion stop (src/getrf2.rs:11)
constexpr int PT = 256;   // threads per CTA in the panel kernel
constexpr int MAXC = 16;  // largest cluster (non-portable size on sm_103)
constexpr size_t SMEM_DATA_LIMIT = 200 * 1024;

struct PanelPub {  // what a CTA publishes to the rest of the cluster each column
  int64_t v;
  int64_t key;
  int64_t g;  // panel row of this CTA's best candidate, -1 if none
  double best_row[PNB];
  double row_j[PNB];  // the current pivot-position row, from the CTA that owns it
};

constexpr size_t panel_base_bytes() {
  return 2 * sizeof(PanelPub) + (PT / 32) * sizeof(Cand) + PNB * sizeof(double) + 4 * sizeof(int64_t) +
         2 * sizeof(double);
}

// Unblocked LU of an mp x nb panel (nb <= 32), iterative_getrf2 of
// src/getrf2.rs:131-185, for panels too tall for the cluster's shared memory:
// the rows stay in global memory (L2), one full cluster barrier per column.
// Panels whose rows fit in shared memory take panel_lu_split below.
__global__ void __launch_bounds__(PT)
panel_lu(double *A, int64_t lda, int64_t mp, int nb, int32_t *ipiv, int32_t *info, int32_t add_on_success,
         int32_t col0, int lanes, int64_t R) {
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int cr = (int)cluster.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PanelPub *pub = reinterpret_cast<PanelPub *>(smem_raw);
  Cand *red = reinterpret_cast<Cand *>(pub + 2);
  double *prow = reinterpret_cast<double *>(red + PT / 32);
  int64_t *bc = reinterpret_cast<int64_t *>(prow + PNB);
  double *pinv = reinterpret_cast<double *>(bc + 4);  // 1 / pivot of the current column

  // Uniform across the cluster: the only writer of *info in this kernel acts
  // after a cluster barrier that every CTA reaches after this read.
  if (stop_flag(info)) return;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t r0 = (int64_t)cr * R;
  const int64_t r1 = imin(mp, r0 + R);
  const int64_t nr = r1 > r0 ? r1 - r0 : 0;
  auto el = [&](int64_t il, int c) -> double & { return A[(r0 + il) + (int64_t)c * lda]; };
  __syncthreads();

  const int steps = (int)imin(mp, nb);
  bool failed = false;
  for (int j = 0; j < steps; ++j) {
    PanelPub *my = &pub[j & 1];
    const int64_t nlen = mp - j;
    // -- idamax over this CTA's rows >= j
    Cand best = cand_none();
    for (int64_t il = tid; il < nr; il += PT) {
      const int64_t g = r0 + il;
      if (g < j) continue;
      const Cand c = make_cand(el(il, j), g - j, nlen, lanes);
      if (cand_better(c, best)) best = c;
    }
    best = warp_best(best);
    if (lane == 0) red[warp] = best;
    __syncthreads();
    if (tid == 0) {
      Cand b = red[0];
      for (int w = 1; w < PT / 32; ++w)
        if (cand_better(red[w], b)) b = red[w];
      my->v = b.v;
      my->key = b.key;
      my->g = (b.v > -2) ? j + b.idx : -1;
      bc[0] = my->g;
    }
    __syncthreads();
    const int64_t myg = bc[0];
    if (tid < nb) {
      if (myg >= 0) my->best_row[tid] = el(myg - r0, tid);
      if (j >= r0 && j < r1) my->row_j[tid] = el(j - r0, tid);
    }
    cluster.sync();
    // -- cluster-wide winner (same total order in every CTA)
    if (warp == 0) {
      Cand c = cand_none();
      if (lane < C) {
        const PanelPub *rp = cluster.map_shared_rank(my, lane);
        c.v = rp->v;
        c.key = rp->key;
        c.idx = rp->g;
      }
      c = warp_best(c);
      if (lane == 0) bc[1] = (c.v < 0) ? (int64_t)j : c.idx;  // idamax -> 0 when nothing qualifies
    }
    __syncthreads();
    const int64_t jp = bc[1];
    const int owner_j = (int)(j / R), owner_p = (int)(jp / R);
    if (tid < nb) {
      const PanelPub *src = cluster.map_shared_rank(my, jp == j ? owner_j : owner_p);
      const double v = (jp == j) ? src->row_j[tid] : src->best_row[tid];
      prow[tid] = v;
      if (tid == j) pinv[0] = 1.0 / v;  // once per CTA, not once per thread
    }
    __syncthreads();
    const double pv = prow[j];
    if (cr == 0 && tid == 0) ipiv[j] = (int32_t)(jp + 1);
    if (!nonzero64(pv)) {  // exact zero pivot: BOLA's "Matrix is singular" (src/getrf2.rs:166-168)
      if (cr == 0 && tid == 0) *info = col0 + j + 1;
      failed = true;
      break;
    }
    // -- row interchange across the whole panel width (src/getrf2.rs:144-150)
    if (jp != j) {
      if (cr == owner_j && tid < nb) el(j - r0, tid) = prow[tid];
      if (cr == owner_p && tid < nb) {
        const PanelPub *sj = cluster.map_shared_rank(my, owner_j);
        el(jp - r0, tid) = sj->row_j[tid];
      }
    }
    __syncthreads();
    // -- reciprocal scale (src/getrf2.rs:152-164) and rank-1 update (ger, src/ger.rs:28-61)
    if (j < mp - 1) {
      const double inv = pinv[0];
      const int64_t mr = mp - j - 1;
      const int64_t rows_vec = (mr / lanes) * lanes;
      const int ncols = nb - j - 1;
      const int n_unrolled = ncols - (ncols % 2);
      const bool do_ger = j < steps - 1;
      for (int64_t il = tid; il < nr; il += PT) {
        const int64_t g = r0 + il;
        if (g <= j) continue;
        const double x = __dmul_rn(el(il, j), inv);
        el(il, j) = x;
        if (!do_ger) continue;
        const bool vec = (g - j - 1) < rows_vec;
        for (int t = 0; t < n_unrolled; t += 2) {
          const int c0 = j + 1 + t;
          const double t0 = -prow[c0], t1 = -prow[c0 + 1];
          if (!nonzero64(t0) && !nonzero64(t1)) continue;
          double &a0 = el(il, c0);
          double &a1 = el(il, c0 + 1);
          a0 = fused_or_unfused(vec, x, t0, a0);
          a1 = fused_or_unfused(vec, x, t1, a1);
        }
        if (ncols % 2) {
          const int c = nb - 1;
          const double t = -prow[c];
          if (nonzero64(t)) el(il, c) = add_prod(el(il, c), t, x);
        }
      }
    }
    __syncthreads();
  }
  if (!failed && cr == 0 && add_on_success != 0)
    for (int t = tid; t < steps; t += PT) ipiv[t] += add_on_success;
  cluster.sync();  // no CTA may leave while another can still read its shared memory
}

// BOLA's rank-1 step (src/getrf2.rs:152-164 with src/ger.rs:28-61) on one
// element: row g (panel row), column c, by pivot p.  x is the row's scaled
// multiplier, prow the pivot row.  ger walks columns p+1.. in pairs, skipping
// a pair whose two pivot-row entries are both zero, with the fused vector
// body for rows below mr rounded down to the SIMD width and the unfused tail
// after; an odd last column is always unfused (and skipped when zero).
struct GerStep {
  int p, nun;       // pivot column, columns of the paired part (ncols rounded down to even)
  int64_t vec_end;  // rows g with g - p - 1 < vec_end take the fused body
};
__device__ __forceinline__ GerStep ger_step(int p, int nb, int64_t mp, int lanes) {
  GerStep s;
  s.p = p;
  s.nun = (nb - p - 1) & ~1;
  s.vec_end = (mp - p - 1) & ~(int64_t)(lanes - 1);
  return s;
}
// -1: the column is skipped, 0: unfused, 1: fused body (rows permitting)
__device__ __forceinline__ int ger_mode(const GerStep &s, const double *prow, int c) {
  const int o = c - s.p - 1;
  if (o < s.nun) {
    const bool any = nonzero64(prow[c]) || nonzero64(prow[s.p + 1 + (o ^ 1)]);
    return any ? 1 : -1;
  }
  return nonzero64(prow[c]) ? 0 : -1;
}
__device__ __forceinline__ double ger_apply(const GerStep &s, int mode, double a, double x, double pc, int64_t g) {
  if (mode < 0) return a;
  const double t = -pc;
  return fused_or_unfused(mode == 1 && g - s.p - 1 < s.vec_end, x, t, a);
}

// What a CTA pushes into every CTA of the cluster for one column: its pivot
// candidate and that row (left before pivot j-1's update of columns > j).
struct XSlot {
  long long v, key, g, pad;  // Cand (g: panel row, -1 if the CTA has none)
  double row[PNB];
};

// The same unblocked LU as panel_lu (BOLA's iterative_getrf2), rows in shared
// memory, with no cluster-wide barrier per column: the candidates travel by
// asynchronous remote stores that count their bytes on the receiver's
// mbarrier (st.async).  Per column j:
//   (a) this CTA's candidate in column j is found (BOLA's lane-ordered idamax
//       keys), one CTA barrier;
//   (b) every warp pushes the CTA's candidate row (and row j, if owned) into
//       its share of the cluster's CTAs, one CTA barrier;
//   (c) the rank-1 update of pivot j-1 on columns j+1.. (deferred), while the
//       pushes land; a bounded wait on this CTA's own mbarrier for all of
//       them (a CTA pushes column j+1 only after it has read column j's
//       slots, which keeps the double-buffered slots and mbarrier phases
//       safe; a push that never lands stops the panel with
//       *info = BOLA_INFO_WAIT_EXPIRED instead of hanging);
//   (d) every CTA picks the same winner from its own slots and brings the
//       pushed rows up to date (the owner's same operation for pivot j-1 on
//       columns > j), one CTA barrier; zero pivot -> stop as BOLA does;
//   (e) the swap, one CTA barrier, the multipliers of column j scaled and the
//       update of column j+1 only (the next column searched).
// Every element sees BOLA's operations in BOLA's order: A, ipiv and info are
// bit-identical to panel_lu's.
__global__ void __launch_bounds__(PT)
panel_lu_split(double *A, int64_t lda, int64_t mp, int nb, int32_t *ipiv, int32_t *info, int32_t add_on_success,
               int32_t col0, int lanes, int64_t R) {
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int cr = (int)cluster.block_rank();
  __shared__ XSlot slots[2][MAXC];
  __shared__ double rowj[2][PNB];
  __shared__ double piv[2][PNB];  // pivot rows, up to date (piv[j & 1] = column j's)
  __shared__ double oldj[PNB];    // the old row j, up to date (goes to the pivot's place)
  __shared__ Cand wc[PT / 32];
  __shared__ double sinv;
  __shared__ uint64_t xbar[2];  // completes when every CTA's push for a column has landed here
  __shared__ int sfail;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *data = reinterpret_cast<double *>(smem_raw);

  // Uniform across the cluster: the only writer of *info here acts after
  // the cluster barrier that every CTA passes after this read.
  if (stop_flag(info)) return;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t r0 = (int64_t)cr * R;
  const int64_t r1 = imin(mp, r0 + R);
  const int64_t nr = r1 > r0 ? r1 - r0 : 0;
  auto el = [&](int c, int64_t il) -> double & { return data[(int64_t)c * R + il]; };
  for (int64_t e = tid; e < nr * nb; e += PT) {
    const int64_t il = e % nr;
    const int c = (int)(e / nr);
    el(c, il) = A[(r0 + il) + (int64_t)c * lda];
  }
  if (tid == 0) {
    sm100::mbar_init(&xbar[0], 1);
    sm100::mbar_init(&xbar[1], 1);
    sm100::fence_mbar_init();
    sfail = 0;
  }
  __syncthreads();
  cluster.sync();  // every CTA runs, its mbarriers initialised, before the first push

  // bytes that land in this CTA per column: a slot (header + row) from every
  // CTA, row j from its owner
  constexpr uint32_t SLOT_BYTES = 3 * 8 + PNB * 8, ROW_BYTES = PNB * 8;
  const uint32_t xbytes = (uint32_t)C * SLOT_BYTES + ROW_BYTES;
  const int steps = (int)imin(mp, nb);
  bool failed = false;
  double inv = 0.0;
  for (int j = 0; j < steps; ++j) {
    const int par = j & 1;
    const double *pprev = piv[par ^ 1];
    // this column's phase of xbar[par] (its previous phase, column j-2, was
    // waited for by every thread): expect the pushes
    if (tid == 0) sm100::mbar_arrive_expect_tx(&xbar[par], xbytes);
    // (a)
    Cand best = cand_none();
    for (int64_t il = tid; il < nr; il += PT) {
      const int64_t g = r0 + il;
      if (g < j) continue;
      const Cand c = make_cand(el(j, il), g - j, mp - j, lanes);
      if (cand_better(c, best)) best = c;
    }
    best = warp_best(best);
    if (lane == 0) wc[warp] = best;
    __syncthreads();
    // (b)
    {
      Cand cb = wc[0];
#pragma unroll
      for (int w = 1; w < PT / 32; ++w)
        if (cand_better(wc[w], cb)) cb = wc[w];
      const int64_t gl = cb.v > -2 ? j + cb.idx - r0 : -1;  // local row of the candidate
      const bool own_j = j >= r0 && j < r1;
      const double cv = (gl >= 0 && lane < nb) ? el(lane, gl) : 0.0;
      const double jv = (own_j && lane < nb) ? el(lane, j - r0) : 0.0;
      for (int d = warp; d < C; d += PT / 32) {
        const uint32_t rbar = sm100::cluster_addr(&xbar[par], d);
        const uint32_t rs = sm100::cluster_addr(&slots[par][cr], d);
        if (lane == 0) {
          sm100::st_async(rs + offsetof(XSlot, v), (long long)cb.v, rbar);
          sm100::st_async(rs + offsetof(XSlot, key), (long long)cb.key, rbar);
          sm100::st_async(rs + offsetof(XSlot, g), (long long)(gl >= 0 ? j + cb.idx : -1), rbar);
        }
        sm100::st_async(rs + (uint32_t)offsetof(XSlot, row) + 8u * lane, cv, rbar);
        if (own_j) sm100::st_async(sm100::cluster_addr(&rowj[par][0], d) + 8u * lane, jv, rbar);
      }
    }
    __syncthreads();  // the rows are read before the deferred update changes them
    // (c) pivot j-1 on columns j+1.., rows >= j
    if (j > 0 && j + 1 < nb && j - 1 < steps - 1) {
      const GerStep gs = ger_step(j - 1, nb, mp, lanes);
      for (int64_t il = tid; il < nr; il += PT) {
        const int64_t g = r0 + il;
        if (g < j) continue;
        const double x = el(j - 1, il);
        for (int c = j + 1; c < nb; ++c) {
          const int mode = ger_mode(gs, pprev, c);
          el(c, il) = ger_apply(gs, mode, el(c, il), x, pprev[c], g);
        }
      }
    }
    // every CTA's push for this column has landed (bounded: a push that
    // never lands stops the panel, never a hang)
    if (!sm100::bounded_wait(&xbar[par], (uint32_t)(j >> 1) & 1u)) sfail = 1;
    __syncthreads();
    if (sfail) {
      if (tid == 0) atomicCAS(info, 0, BOLA_INFO_WAIT_EXPIRED);
      failed = true;
      break;
    }
    // (d) the winner, identical in every CTA
    Cand wk = cand_none();
    int ws = 0;
    {
      Cand k = cand_none();
      if (lane < C) {
        k.v = slots[par][lane].v;
        k.key = slots[par][lane].key;
        k.idx = slots[par][lane].g;
      }
      wk = warp_best(k);
      wk.v = __shfl_sync(0xffffffffu, wk.v, 0);
      wk.key = __shfl_sync(0xffffffffu, wk.key, 0);
      wk.idx = __shfl_sync(0xffffffffu, wk.idx, 0);
      const unsigned m = __ballot_sync(0xffffffffu, lane < C && k.v == wk.v && k.key == wk.key && k.idx == wk.idx);
      ws = m ? __ffs(m) - 1 : 0;
    }
    const int64_t jp = wk.v < 0 ? (int64_t)j : wk.idx;  // idamax -> 0 when nothing qualifies
    const double *raw = jp == j ? rowj[par] : slots[par][ws].row;
    double *pcur = piv[par];
    if (tid < nb) {
      double pv_ = raw[tid], ov = rowj[par][tid];
      if (j > 0 && tid > j && j - 1 < steps - 1) {
        const GerStep gs = ger_step(j - 1, nb, mp, lanes);
        const int mode = ger_mode(gs, pprev, tid);
        pv_ = ger_apply(gs, mode, pv_, raw[j - 1], pprev[tid], jp);
        ov = ger_apply(gs, mode, ov, rowj[par][j - 1], pprev[tid], j);
      }
      pcur[tid] = pv_;
      oldj[tid] = ov;
      if (tid == j) sinv = 1.0 / pv_;  // once per CTA
    }
    __syncthreads();
    const double pv = pcur[j];
    if (cr == 0 && tid == 0) ipiv[j] = (int32_t)(jp + 1);
    if (!nonzero64(pv)) {  // exact zero pivot: BOLA's "Matrix is singular" (src/getrf2.rs:166-168)
      if (cr == 0 && tid == 0) *info = col0 + j + 1;
      failed = true;
      break;
    }
    inv = sinv;
    // (e)
    if (jp != j && tid < nb) {
      if (j >= r0 && j < r1) el(tid, j - r0) = pcur[tid];
      if (jp >= r0 && jp < r1) el(tid, jp - r0) = oldj[tid];
    }
    __syncthreads();
    if (j < mp - 1) {
      const bool next = j + 1 < nb && j < steps - 1;
      const GerStep gs = ger_step(j, nb, mp, lanes);
      const int mode = next ? ger_mode(gs, pcur, j + 1) : -1;
      for (int64_t il = tid; il < nr; il += PT) {
        const int64_t g = r0 + il;
        if (g <= j) continue;
        const double x = __dmul_rn(el(j, il), inv);
        el(j, il) = x;
        if (next) el(j + 1, il) = ger_apply(gs, mode, el(j + 1, il), x, pcur[j + 1], g);
      }
    }
  }
  if (!failed && cr == 0 && add_on_success != 0)
    for (int t = tid; t < steps; t += PT) ipiv[t] += add_on_success;
  __syncthreads();
  for (int64_t e = tid; e < nr * nb; e += PT) {
    const int64_t il = e % nr;
    const int c = (int)(e / nr);
    A[(r0 + il) + (int64_t)c * lda] = el(c, il);
  }
  cluster.sync();  // no CTA may leave while another can still read its shared memory
}

// iterative_getrf2 for a short, wide matrix (m <= 32 rows, any n): one CTA,
// data in global memory.
__global__ void __launch_bounds__(PT)
panel_lu_wide(double *A, int64_t lda, int64_t m, int64_t n, int32_t *ipiv, int32_t *info, int32_t col0,
              int lanes) {
  __shared__ Cand red[PT / 32];
  __shared__ int64_t sjp;
  if (stop_flag(info)) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t steps = imin(m, n);
  for (int64_t j = 0; j < steps; ++j) {
    Cand best = cand_none();
    for (int64_t g = j + tid; g < m; g += PT) {
      const Cand c = make_cand(A[g + j * lda], g - j, m - j, lanes);
      if (cand_better(c, best)) best = c;
    }
    best = warp_best(best);
    if (lane == 0) red[warp] = best;
    __syncthreads();
    if (tid == 0) {
      Cand b = red[0];
      for (int w = 1; w < PT / 32; ++w)
        if (cand_better(red[w], b)) b = red[w];
      sjp = (b.v < 0) ? j : j + b.idx;
      ipiv[j] = (int32_t)(sjp + 1);
    }
    __syncthreads();
    const int64_t jp = sjp;
    const double pv = A[jp + j * lda];
    if (!nonzero64(pv)) {
      if (tid == 0) *info = col0 + (int32_t)j + 1;
      return;
    }
    if (jp != j) {
      for (int64_t c = tid; c < n; c += PT) {
        const double t = A[j + c * lda];
        A[j + c * lda] = A[jp + c * lda];
        A[jp + c * lda] = t;
      }
    }
    __syncthreads();
    if (j < m - 1) {
      const double inv = 1.0 / pv;
      for (int64_t g = j + 1 + tid; g < m; g += PT) A[g + j * lda] = __dmul_rn(A[g + j * lda], inv);
    }
    __syncthreads();
    if (j < steps - 1) {
      const int64_t mr = m - j - 1, ncols = n - j - 1;
      const int64_t rows_vec = (mr / lanes) * lanes, n_unrolled = ncols - (ncols % 2);
      for (int64_t e = tid; e < mr * ncols; e += PT) {
        const int64_t ri = e % mr, ci = e / mr;
        const int64_t g = j + 1 + ri, c = j + 1 + ci;
        const double x = A[g + j * lda];
        double &a = A[g + c * lda];
        if (ci < n_unrolled) {
          const int64_t p0 = j + 1 + (ci & ~(int64_t)1);
          const double t0 = -A[j + p0 * lda], t1 = -A[j + (p0 + 1) * lda];
          if (!nonzero64(t0) && !nonzero64(t1)) continue;
          const double t = (c == p0) ? t0 : t1;
          a = fused_or_unfused(ri < rows_vec, x, t, a);
        } else {
          const double t = -A[j + c * lda];
          if (nonzero64(t)) a = add_prod(a, t, x);
        }
      }
    }
    __syncthreads();
  }
}

// One getrf block step after the panel: the panel's interchanges applied to
// all other columns (src/getrf.rs:64-70) and, on the right block row, BOLA's
// unit-lower trsm base case with its daxpy (src/getrf.rs:78, src/trsm.rs:96-109).
// A warp per column.
__global__ void __launch_bounds__(256)
step_swap_trsm(double *A, int64_t lda, int64_t n, int64_t j, int jb, const int32_t *ipiv,
               const int32_t *info, int lanes) {
  __shared__ int64_t rows[2 * PNB], src[2 * PNB];
  __shared__ double L[PNB * PNB];
  __shared__ int cnt;
  if (stop_flag(info)) return;
  if (threadIdx.x < 32) {
    SwapPlan p;
    p.ix0 = j;
    p.i1 = (int32_t)(j + 1);
    p.i2 = (int32_t)(j + jb);
    p.i_inc = 1;
    p.incx = 1;
    const int c = compose_swaps_warp(p, ipiv, rows, src);
    if (threadIdx.x == 0) cnt = c;
  }
  for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) {
    const int r = e % jb, c = e / jb;
    L[r + c * PNB] = A[(j + r) + (j + c) * lda];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= n - jb) return;
  const int64_t col = w < j ? w : w + jb;
  double *cp = A + col * lda;
  const double v0 = lane < cnt ? cp[src[lane]] : 0.0;
  const double v1 = lane + 32 < cnt ? cp[src[lane + 32]] : 0.0;
  __syncwarp();
  if (lane < cnt) cp[rows[lane]] = v0;
  if (lane + 32 < cnt) cp[rows[lane + 32]] = v1;
  __syncwarp();
  if (col < j + jb) return;
  double b = lane < jb ? cp[j + lane] : 0.0;
  for (int k = 0; k < jb; ++k) {
    const double bk = __shfl_sync(0xffffffffu, b, k);
    if (!nonzero64(bk)) continue;
    if (lane > k && lane < jb)
      b = daxpy_elem(b, -bk, L[lane + k * PNB], lane - k - 1, jb - k - 1, lanes);
  }
  if (lane < jb) cp[j + lane] = b;
}

__global__ void zero_i32(int32_t *p) { *p = 0; }
__global__ void copy_i32(const int32_t *src, int32_t *dst) { *dst = *src; }

// Launches panel_lu with the largest cluster (<= 16 CTAs, ~256 rows each)
// the device can co-schedule.
int launch_panel(cudaStream_t s, double *A, int64_t lda, int64_t mp, int nb, int32_t *ipiv, int32_t *info,
                 int32_t add_on_success, int32_t col0) {
  double fl = 0.0;
  for (int j = 0; j < nb && j < mp; ++j) fl += (double)(mp - j - 1) * (1.0 + 2.0 * (nb - j - 1));
  ProfScope prof(s, "getrf_panel", fl, 16.0 * (double)mp * nb);
  int C = (int)imin(MAXC, imax(1, cdiv(mp, 256)));
  for (;; C = C > 1 ? (C + 1) / 2 : 0) {
    if (C == 0) return fail(BOLA_ERR_CUDA, "panel_lu: no cluster size could be scheduled");
    const int64_t R = cdiv(mp, C);
    // rows in shared memory: the split-barrier kernel; taller panels keep
    // their rows in global memory (panel_lu)
    const size_t rows_bytes = (size_t)R * nb * sizeof(double);
    const bool use_smem = rows_bytes <= SMEM_DATA_LIMIT;
    const size_t smem = use_smem ? rows_bytes : panel_base_bytes();
    void (*kern)(double *, int64_t, int64_t, int, int32_t *, int32_t *, int32_t, int32_t, int, int64_t) =
        use_smem ? panel_lu_split : panel_lu;
    BOLA_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_DATA_LIMIT + 4096));
    BOLA_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C, 1, 1);
    cfg.blockDim = dim3(PT, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      continue;
    }
    const int lanes_v = lanes();
    BOLA_TRY_CUDA(cudaLaunchKernelEx(&cfg, kern, A, lda, mp, nb, ipiv, info, add_on_success, col0, lanes_v, R));
    return 0;
  }
}

// iterative_getrf2 dispatch: tall panels go to the cluster kernel, short wide
// ones to the single-CTA kernel.
int iterative(cudaStream_t s, int64_t m, int64_t n, double *A, int64_t lda, int32_t *ipiv, int32_t *info,
              int32_t col0, int32_t add_on_success) {
  if (n <= PNB) return launch_panel(s, A, lda, m, (int)n, ipiv, info, add_on_success, col0);
  ProfScope prof(s, "getrf_panel_wide", 2.0 * (double)m * m * n);
  panel_lu_wide<<<1, PT, 0, s>>>(A, lda, m, n, ipiv, info, col0, lanes());
  BOLA_CHECK_LAUNCH();
  return ipiv_add(s, ipiv, imin(m, n), add_on_success, info);
}

}  // namespace

// src/getrf2.rs:39-106; col0 is the global column of A's first column (for info).
int getrf2_rec(cudaStream_t s, int64_t m, int64_t n, double *A, int64_t lda, int32_t *ipiv, int32_t *info,
               int32_t col0) {
  if (m == 0 || n == 0) return 0;
  if (m <= PNB || n <= PNB) return iterative(s, m, n, A, lda, ipiv, info, col0, 0);
  const int64_t n1 = imin(m, n) / 2, n2 = n - n1;
  BOLA_TRY(getrf2_rec(s, m, n1, A, lda, ipiv, info, col0));
  BOLA_TRY(laswp_exact(s, n2, A + n1 * lda, lda, 1, (int32_t)n1, ipiv, 1, info));
  BOLA_TRY(trsm_exact(s, 'L', 'L', 'N', 'U', n1, n2, 1.0, A, lda, A + n1 * lda, lda, info));
  if (n1 < m) {
    BOLA_TRY(dgemm_exact(s, 'N', 'N', m - n1, n2, n1, -1.0, A + n1, lda, A + n1 * lda, lda, 1.0,
                         A + n1 + n1 * lda, lda, 64, info, 0));
    BOLA_TRY(getrf2_rec(s, m - n1, n2, A + n1 + n1 * lda, lda, ipiv + n1, info, col0 + (int32_t)n1));
  }
  BOLA_TRY(ipiv_add(s, ipiv + n1, imin(m, n) - n1, (int32_t)n1, info));
  return laswp_exact(s, n1, A, lda, (int32_t)(n1 + 1), (int32_t)imin(m, n), ipiv, 1, info);
}

// src/getrf.rs:37-101

// ---- look-ahead stream pool (shared by the blocked getrf and potrf) ----------
namespace {
std::mutex g_la_mu;
std::vector<LookAhead *> g_la_pool[64];
}  // namespace

LookAhead *la_acquire() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  {
    std::lock_guard<std::mutex> lk(g_la_mu);
    auto &pool = g_la_pool[dev & 63];
    if (!pool.empty()) {
      LookAhead *la = pool.back();
      pool.pop_back();
      return la;
    }
  }
  LookAhead *la = new LookAhead();
  int least = 0, greatest = 0;
  bool ok = cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess &&
            cudaStreamCreateWithPriority(&la->sp, cudaStreamNonBlocking, greatest) == cudaSuccess &&
            cudaStreamCreateWithPriority(&la->su, cudaStreamNonBlocking, least) == cudaSuccess &&
            cudaMalloc(&la->snap, 2 * sizeof(int32_t)) == cudaSuccess;
  for (cudaEvent_t &e : la->ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) return nullptr;  // (leaks the partial set; only on a failing device)
  return la;
}

void la_release(LookAhead *la) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_la_mu);
  g_la_pool[dev & 63].push_back(la);
}

// BOLA's blocked getrf (src/getrf.rs:37-101) with look-ahead.  Per step k:
// panel, swaps + trsm, and the update of the next panel's 32 columns on sp;
// the update of the other columns on su, overlapping panel k+1 (whose swaps
// wait for it).  Splitting the trailing DGEMM at a column multiple of 4 keeps
// BOLA's 8x4 edge-tile classification, so every element is computed exactly
// as in one call.  The wide update stops on its own step's snapshot of
// *info: a zero pivot found by panel k+1 while it runs must not cut short
// step k's update, which BOLA completes before factoring panel k+1.
int getrf_blocked(cudaStream_t s, int64_t m, int64_t n, double *A, int64_t lda, int32_t *ipiv, int32_t *info) {
  const int64_t min_mn = imin(m, n);
  // look-ahead pays from a few hundred columns on; below that its events and
  // the extra launches cost more than the overlap saves
  LookAhead *la = (m > 0 && n > 0 && min_mn >= 512) ? la_acquire() : nullptr;
  if (!la) {
    {
      ProfScope prof(s, "info_init");
      zero_i32<<<1, 1, 0, s>>>(info);
    }
    BOLA_CHECK_LAUNCH();
    if (m == 0 || n == 0) return 0;
    if (PNB >= min_mn) return getrf2_rec(s, m, n, A, lda, ipiv, info, 0);
    for (int64_t j = 0; j < min_mn; j += PNB) {
      const int jb = (int)imin(PNB, min_mn - j);
      BOLA_TRY(launch_panel(s, A + j + j * lda, lda, m - j, jb, ipiv + j, info, (int32_t)j, (int32_t)j));
      const int64_t others = n - jb;
      if (others > 0) {
        ProfScope prof(s, "getrf_swap_trsm", (double)jb * (jb - 1) * (double)(n - j - jb), 32.0 * jb * (double)others);
        step_swap_trsm<<<(unsigned)cdiv(others, 8), 256, 0, s>>>(A, lda, n, j, jb, ipiv, info, lanes());
        BOLA_CHECK_LAUNCH();
      }
      if (j + jb < n && j + jb < m) {
        BOLA_TRY(dgemm_exact(s, 'N', 'N', m - j - jb, n - j - jb, jb, -1.0, A + (j + jb) + j * lda, lda,
                             A + j + (j + jb) * lda, lda, 1.0, A + (j + jb) + (j + jb) * lda, lda, 64, info, 0));
      }
    }
    return 0;
  }
  int st = 0;
  auto run = [&]() -> int {
    BOLA_TRY_CUDA(cudaEventRecord(la->ev[0], s));
    BOLA_TRY_CUDA(cudaStreamWaitEvent(la->sp, la->ev[0], 0));
    BOLA_TRY_CUDA(cudaStreamWaitEvent(la->su, la->ev[0], 0));
    {
      ProfScope prof(la->sp, "info_init");
      zero_i32<<<1, 1, 0, la->sp>>>(info);
    }
    BOLA_CHECK_LAUNCH();
    bool wide_pending = false;
    for (int64_t j = 0, k = 0; j < min_mn; j += PNB, ++k) {
      const int jb = (int)imin(PNB, min_mn - j);
      BOLA_TRY(launch_panel(la->sp, A + j + j * lda, lda, m - j, jb, ipiv + j, info, (int32_t)j, (int32_t)j));
      if (wide_pending) BOLA_TRY_CUDA(cudaStreamWaitEvent(la->sp, la->ev[2], 0));
      wide_pending = false;
      const int64_t others = n - jb;
      if (others > 0) {
        ProfScope prof(la->sp, "getrf_swap_trsm", (double)jb * (jb - 1) * (double)(n - j - jb),
                       32.0 * jb * (double)others);
        step_swap_trsm<<<(unsigned)cdiv(others, 8), 256, 0, la->sp>>>(A, lda, n, j, jb, ipiv, info, lanes());
        BOLA_CHECK_LAUNCH();
      }
      if (!(j + jb < n && j + jb < m)) continue;
      const int64_t m2 = m - j - jb, n2 = n - j - jb;
      const int64_t nb_next = imin((int64_t)PNB, n2);  // a multiple of 4 unless it is all of n2
      const double *A21 = A + (j + jb) + j * lda, *A12 = A + j + (j + jb) * lda;
      double *A22 = A + (j + jb) + (j + jb) * lda;
      BOLA_TRY(dgemm_exact(la->sp, 'N', 'N', m2, nb_next, jb, -1.0, A21, lda, A12, lda, 1.0, A22, lda, 64, info, 0));
      if (n2 > nb_next) {
        int32_t *snap = la->snap + (k & 1);
        copy_i32<<<1, 1, 0, la->sp>>>(info, snap);
        BOLA_CHECK_LAUNCH();
        BOLA_TRY_CUDA(cudaEventRecord(la->ev[1], la->sp));
        BOLA_TRY_CUDA(cudaStreamWaitEvent(la->su, la->ev[1], 0));
        BOLA_TRY(dgemm_exact(la->su, 'N', 'N', m2, n2 - nb_next, jb, -1.0, A21, lda, A12 + nb_next * lda, lda, 1.0,
                             A22 + nb_next * lda, lda, 64, snap, 0));
        BOLA_TRY_CUDA(cudaEventRecord(la->ev[2], la->su));
        wide_pending = true;
      }
    }
    if (wide_pending) BOLA_TRY_CUDA(cudaStreamWaitEvent(la->sp, la->ev[2], 0));
    BOLA_TRY_CUDA(cudaEventRecord(la->ev[3], la->sp));
    BOLA_TRY_CUDA(cudaStreamWaitEvent(s, la->ev[3], 0));
    return 0;
  };
  st = run();
  if (st != 0) {
    // leave nothing of this call running on the look-ahead streams
    cudaStreamSynchronize(la->sp);
    cudaStreamSynchronize(la->su);
  }
  la_release(la);
  return st;
}

}  // namespace bola

using namespace bola;

extern "C" {

int bola_dgetrf(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv, int32_t *info,
                bola_stream_t stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (lda < imax(m, 1)) return -4;  // "Argument 4 to getrf had an illegal value" (src/getrf.rs:41-43)
  if (imin(m, n) > INT32_MAX - 1) return -1;
  if (info == nullptr) return -6;
  return getrf_blocked((cudaStream_t)stream, m, n, a, lda, ipiv, info);
}

int bola_dgetrf2(int64_t m, int64_t n, double *a, int64_t lda, int32_t *ipiv, int32_t *info,
                 bola_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (lda < imax(m, 1)) return -4;  // src/getrf2.rs:43-45
  if (info == nullptr) return -6;
  {
    ProfScope prof(s, "info_init");
    zero_i32<<<1, 1, 0, s>>>(info);
  }
  BOLA_CHECK_LAUNCH();
  return getrf2_rec(s, m, n, a, lda, ipiv, info, 0);
}

int bola_dgetrs(int64_t n, int64_t nrhs, const double *lu, int64_t lda, const int32_t *ipiv, double *b,
                int64_t ldb, bola_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (lda < imax(1, n)) return -4;
  if (ldb < imax(1, n)) return -7;
  if (n == 0 || nrhs == 0) return 0;
  BOLA_TRY(laswp_exact(s, nrhs, b, ldb, 1, (int32_t)n, ipiv, 1, nullptr));
  BOLA_TRY(trsm_exact(s, 'L', 'L', 'N', 'U', n, nrhs, 1.0, lu, lda, b, ldb, nullptr));
  return trsm_exact(s, 'L', 'U', 'N', 'N', n, nrhs, 1.0, lu, lda, b, ldb, nullptr);
}

}  // extern "C"
