// slu.cu — the low-precision LU of the mixed-precision solver (no BOLA
// counterpart; it preconditions the FP64 refinement in ir.cu).
//
// A (FP64) is scaled per 64-column block by a power of two (exact) and
// rounded to the working matrix W: FP32 (factor kinds 0-2) or FP64 (kind 3).
// Blocked right-looking LU, NB = 64 = the K of the tensor-core update:
//   tpanel_kernel   FP32 W: the (n-j) x 64 panel on a cluster of <= 16 CTAs,
//                   rows in shared memory, pivots chosen by tournament over
//                   groups of 8 columns (one cluster exchange per group);
//                   writes L21 as the update's K-major A operand (bf16 or
//                   tf32 hi/lo).
//   FP64 W (the FP64-accurate factor): the same tournament on FP32 copies
//                   chooses the pivot rows (tpanel_kernel<double>), then
//                   panel_lu64 factors the panel in FP64 in that pivot order
//                   on as many SMs as it has 64-row slices, writing L21's
//                   exact bf16 slices as the A operand.
//   sswap_trsm      the 64 interchanges on the columns right of the panel,
//                   U12 = L11^-1 A12 and the K-major B operand (the columns
//                   left of it take them at the end: apply_left_swaps).
//   tc_update / oz_update   W22 -= L21 U12 on tcgen05 (tc_update.cu, oz_update.cu).
// Pivots are this algorithm's own; only the FP64 refinement decides accuracy.
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <type_traits>

#include "common.cuh"
#include "mixed.cuh"
#include "sm100.cuh"

namespace cg = cooperative_groups;

namespace bola {
namespace {

constexpr int SNB = 64;   // panel width and update depth
constexpr int SMAXC = 16;
// a panel's moves of rows for the swap kernels: count, rows[128], src[128] (+ spare)
constexpr int PLAN_STRIDE = 1 + 4 * SNB;

// Bulk copy of `bytes` (a multiple of 16) from this CTA's shared memory into
// another CTA's (cluster addresses dst and bar), completing on the
// receiver's mbarrier; the issuing thread commits it as a bulk group.
__device__ __forceinline__ void bulk_push(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "r"(sm100::smem_u32(src)), "r"(bytes), "r"(bar)
      : "memory");
}

// Row pitch of a panel held in shared memory: at least R + 1 and a multiple
// of the 16-byte vector (4 floats or 2 doubles), so that a lane can move V
// consecutive rows of a column in one access.
template <typename T>
__host__ __device__ constexpr int panel_pitch(int64_t R) {
  return (int)(((R + (int64_t)(16 / sizeof(T))) / (int64_t)(16 / sizeof(T))) * (int64_t)(16 / sizeof(T)));
}

// ---- tournament panel (the FP32 factors; pivot selection of the FP64 one) ----------------------------------------
// Partial pivoting exchanges the pivot candidates of every CTA once per
// column, so a cluster panel pays 64 cluster round trips.  The FP32 factors
// (kinds 0-2) select their pivots by tournament instead (TSLU, the panel
// step of communication-avoiding LU): per group of TG = 8 columns,
//   1. every warp runs partial pivoting on its own rows over the group's
//      columns (in registers, on scratch copies) and nominates TG rows;
//   2. warp 0 runs it again on the CTA's 8 x TG nominees (their current
//      values, not the warps' eliminated copies) and keeps TG;
//   3. each CTA pushes its TG nominees into every CTA's shared memory
//      (st.async onto the receiver's mbarrier: one exchange per group instead
//      of one per column);
//   4. while the pushes fly, each CTA applies the previous group's update to
//      its rows' columns right of the current group (look-ahead: the previous
//      group only updated the current group's columns before the search);
//   5. every CTA runs partial pivoting on the same C x TG stacked nominees and
//      so picks the same TG pivot rows, with their multipliers; the pivots' U
//      rows right of the group come from the pushed rows, brought up to date
//      with the previous group's update first (the pushed multipliers of that
//      group travel with them);
//   6. every CTA gives its rows the group's multipliers (forward substitution
//      through the TG x TG block of U) and updates the next group's columns.
// Rows never move during the panel (a per-row state records which column a
// row is the pivot of); the interchanges (LAPACK ipiv) are derived at the end
// and every row is written back once, to its final position.  The pivots are
// not those of column-by-column partial pivoting; their growth is that of
// tournament pivoting (CALU), and only the FP64 refinement decides accuracy.
constexpr int TG = 8;     // columns per tournament group
constexpr int TPT = 256;  // threads per panel CTA (8 warps)
constexpr int TRPL = 2;   // panel rows per thread: R <= TPT * TRPL = 512

struct alignas(16) TSlot {
  uint32_t row, pad0, pad1, pad2;  // panel row of the nominee, or 0xFFFFFFFF (none)
  float v[SNB];                    // its values from column pb on: v[k] = column pb + k
};

// Partial pivoting over gw <= TG columns of candidates held by the first NW
// warps of the CTA: thread t (< 32 NW) holds candidate t + 32 NW r in row r
// of v (r < RPL), the current column always in register slot 0 (the others
// shift down after each step, which keeps the column loop rolled).  Pivot
// key: |v| with its KB lowest bits replaced by (2^KB - 1 - candidate), so a
// warp reduction and a maximum over the NW warps' results find the pivot
// (the lowest mantissa bits do not matter for the pivot's quality; ties go
// to the lowest candidate; a NaN never wins over a number).  Per step: the
// warps' maxima meet in shared memory at one named barrier over the NW
// warps, the pivot's owner publishes its row at a second, and every thread
// updates its own candidates.  Writes the selected candidates in order to
// sel[] and returns their count (the same in every thread).  RECORD: each
// candidate's multipliers go to Lsm[candidate * TG + step], the selected
// rows' ones to Lrec[t][s] (s < t), and the pivot rows' eliminated values in
// group column t + k to Urec[(t + k) * uk + t].
template <int RPL, int NW, bool RECORD>
__device__ __forceinline__ int group_gepp(float (&v)[RPL][TG], bool (&live)[RPL], int gw, int32_t *sel, int bar,
                                          uint32_t *wmax, float *prow, float *Lsm, float (*Lrec)[TG], float *Urec,
                                          int uk) {
  constexpr int NT = 32 * NW;
  constexpr uint32_t MASK = RPL * NT <= 256 ? 0xFFu : 0x3FFu;  // candidate-index bits
  static_assert(RPL * NT <= 1024, "too many candidates for the key");
  const int t0 = threadIdx.x, lane = t0 & 31, w = t0 >> 5;
  int cnt = 0;
#pragma unroll 1
  for (int t = 0; t < gw; ++t) {
    uint32_t key = 0u;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const float x = fabsf(v[r][0]);
      const uint32_t a = x == x ? __float_as_uint(x) : 0u;
      const uint32_t k = (a & ~MASK) | (MASK - (uint32_t)(t0 + NT * r));
      key = (live[r] && k > key) ? k : key;
    }
    key = __reduce_max_sync(0xffffffffu, key);
    if (lane == 0) wmax[w] = key;
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(NT) : "memory");
    uint32_t mk = wmax[0];
#pragma unroll
    for (int i = 1; i < NW; ++i) mk = wmax[i] > mk ? wmax[i] : mk;
    if (mk == 0u) break;  // no live candidate left (a live one has a key > 0)
    const int ci = (int)(MASK - (mk & MASK));
    if (t0 == ci % NT) {  // the owner publishes the pivot row and retires it
      const int ro = ci / NT;
#pragma unroll
      for (int r = 0; r < RPL; ++r)
        if (r == ro) {
#pragma unroll
          for (int k = 0; k < TG; ++k) prow[k] = v[r][k];
          live[r] = false;
        }
      sel[t] = ci;
    }
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(NT) : "memory");
    float pv[TG];
#pragma unroll
    for (int k = 0; k < TG; ++k) pv[k] = prow[k];
    if (RECORD) {
      if (t0 < t) Lrec[t][t0] = Lsm[ci * TG + t0];
      if (t0 < TG && t0 < gw - t) Urec[(t + t0) * uk + t] = pv[t0];
    }
    const float inv = pv[0] != 0.f ? __frcp_rn(pv[0]) : 0.f;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const float l = v[r][0] * inv;
      if (RECORD && live[r]) Lsm[(t0 + NT * r) * TG + t] = l;
#pragma unroll
      for (int k = 1; k < TG; ++k) v[r][k - 1] = live[r] ? fmaf(-l, pv[k], v[r][k]) : v[r][k];
      v[r][TG - 1] = 0.f;
    }
    ++cnt;
  }
  return cnt;
}

// LAPACK's interchanges for a panel whose pivot of column j is panel row x
// (j < jb), one column at a time in column order: interchange_step returns
// ipiv's entry for column j (col0 + 1 + the position row j swaps with).  Rows
// below the panel's first jb never move until they become a pivot; rows among
// the first jb are tracked: at_[q] = the row now in position q < jb,
// posin[x] = the position of original row x < jb (interchanges_init: the
// identity).  One thread; a column's step needs only the pivots before it, so
// the kernels run the steps while the later columns are still being factored.
__device__ __forceinline__ void interchanges_init(int jb, int32_t *posin, int32_t *at_) {
  for (int x = 0; x < jb; ++x) posin[x] = at_[x] = x;
}
__device__ __forceinline__ int32_t interchange_step(int j, int x, int jb, int32_t col0, int32_t *posin,
                                                    int32_t *at_) {
  const int q = x < jb ? posin[x] : x;
  const int r = at_[j];
  if (r != x) {
    if (q < jb) at_[q] = r;
    posin[r] = q;
  }
  at_[j] = x;
  if (x < jb) posin[x] = j;
  return col0 + q + 1;
}

// The panel's row interchanges as "row rows[t] takes the old row src[t]"
// (global rows) for the swap kernel: plan[0] = count, then rows, then src.
// From the final state of the interchange steps (no replay of the swaps):
// position q < jb takes its pivot pivl[q], and each of the first jb rows
// that is not a pivot goes to the position posin[x] >= jb it was displaced
// to.  One warp; entries are compacted with ballots.  With rows_s != nullptr
// the list also goes to shared memory, as panel rows (rows_s, src_s, *cnt_s).
__device__ __forceinline__ void list_panel_moves(const int32_t *pivl, const int32_t *posin, int jb, int32_t col0,
                                                 int32_t *plan, int32_t *rows_s = nullptr, int32_t *src_s = nullptr,
                                                 int *cnt_s = nullptr) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int base = 0;
  for (int q0 = 0; q0 < jb; q0 += 32) {
    const int q = q0 + lane;
    const bool mv = q < jb && pivl[q] != q;
    const unsigned m = __ballot_sync(FULL, mv);
    if (mv) {
      const int slot = base + __popc(m & ((1u << lane) - 1u));
      plan[1 + slot] = col0 + q;
      plan[1 + 2 * SNB + slot] = col0 + pivl[q];
      if (rows_s != nullptr) {
        rows_s[slot] = q;
        src_s[slot] = pivl[q];
      }
    }
    base += __popc(m);
  }
  for (int x0 = 0; x0 < jb; x0 += 32) {
    const int x = x0 + lane;
    const bool mv = x < jb && posin[x] >= jb;
    const unsigned m = __ballot_sync(FULL, mv);
    if (mv) {
      const int slot = base + __popc(m & ((1u << lane) - 1u));
      plan[1 + slot] = col0 + posin[x];
      plan[1 + 2 * SNB + slot] = col0 + x;
      if (rows_s != nullptr) {
        rows_s[slot] = posin[x];
        src_s[slot] = x;
      }
    }
    base += __popc(m);
  }
  if (lane == 0) {
    plan[0] = base;
    if (cnt_s != nullptr) *cnt_s = base;
  }
}

// Dynamic shared memory of the tournament panel: the rows (column-major,
// pitch RP, 64 columns, zero beyond jb), the double-buffered nominee slots
// (C x TG per buffer) and the row states.
__host__ __device__ constexpr size_t tpanel_smem(int64_t R, int C) {
  return sizeof(float) * (size_t)SNB * (size_t)panel_pitch<float>(R) + 2 * (size_t)C * TG * sizeof(TSlot) +
         sizeof(int16_t) * (size_t)(R + 8);
}

// a -= sum_s l[s] u[s] (s = 0..7, in order)
__device__ __forceinline__ float rank8(float a, const float (&l)[TG], const float4 &u0, const float4 &u1) {
  a = fmaf(-l[0], u0.x, a);
  a = fmaf(-l[1], u0.y, a);
  a = fmaf(-l[2], u0.z, a);
  a = fmaf(-l[3], u0.w, a);
  a = fmaf(-l[4], u1.x, a);
  a = fmaf(-l[5], u1.y, a);
  a = fmaf(-l[6], u1.z, a);
  a = fmaf(-l[7], u1.w, a);
  return a;
}

// G = float: the FP32 factors' panel (factored in place).  G = double: the
// FP64-accurate factor's pivot selection only — the tournament runs on FP32
// copies of the panel's values and writes the jb pivot rows (panel rows, in
// column order) to winout and their FP64 values (columns of the panel) to
// sel, 64 x 64 row-major; W, ipiv, info and the operands are left to the
// FP64 kernel that follows (panel_lu64).
template <typename G>
__global__ void __launch_bounds__(TPT, 1)
tpanel_kernel(G *W, int64_t ldw, int64_t mp, int jb, int32_t *ipiv, int32_t col0, int32_t *info, int64_t R,
              int32_t *plan, uint64_t *track, double give_up, int32_t *err, int32_t *winout, G *sel) {
  constexpr bool SEL = std::is_same<G, double>::value;
  sm100::grid_dependency_wait();
  cg::cluster_group cluster = cg::this_cluster();
  // an abandoned factorisation (flag set by an earlier panel on this stream,
  // so every CTA reads the same value): identity pivots keep ipiv valid
  if (track != nullptr && *(volatile const int32_t *)(track + 2) != 0) {
    if (cluster.block_rank() == 0)
      for (int t = threadIdx.x; t < jb; t += blockDim.x) ipiv[t] = col0 + t + 1;
    return;
  }
  const int C = (int)cluster.num_blocks();
  const int cr = (int)cluster.block_rank();
  __shared__ uint64_t xbar[2];             // completes when every CTA's nominees of a group have landed
  __shared__ int32_t cand2[TG];            // the CTA's nominees (local rows, -1: none)
  __shared__ uint32_t gwmax[TPT / 32];     // pivot searches: the warps' best keys
  __shared__ float gprow[TG];              // pivot searches: the pivot row of the current step
  __shared__ int32_t win[SNB];             // panel row of the pivot of each column
  __shared__ int32_t wslot[TG];            // the group's pivots as slot indices
  __shared__ float Lg[TG][TG];             // the group pivots' multipliers within the group
  __shared__ __align__(16) float UgT[2][SNB][TG];  // U rows of a group's pivots, transposed (two groups)
  __shared__ float invp[TG];
  __shared__ int32_t posin[SNB], at_[SNB];  // interchange bookkeeping (CTA 0)
  __shared__ int sfail;
  __shared__ TSlot stage[TG];              // this CTA's nominees, as they are pushed
  __shared__ int32_t selw[2][TG];          // pivot searches' outputs (candidate order): own rows, nominees
  __shared__ float Lsm[SMAXC * TG * TG];   // multipliers of the stacked nominees, per step
  __shared__ float Linv[TG][TG];           // inverse of the group's unit-lower 8 x 8 block of L
  extern __shared__ __align__(16) unsigned char tp_raw[];
  const int RP = panel_pitch<float>(R);
  float *sp = reinterpret_cast<float *>(tp_raw);
  TSlot *slots = reinterpret_cast<TSlot *>(tp_raw + sizeof(float) * (size_t)SNB * RP);
  int16_t *rstate = reinterpret_cast<int16_t *>(tp_raw + sizeof(float) * (size_t)SNB * RP +
                                                2 * (size_t)C * TG * sizeof(TSlot));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = (int)(cr * R);
  const int r1 = (int)imin(mp, r0 + R);
  const int nr = r1 > r0 ? r1 - r0 : 0;

  // the panel into shared memory: a thread's rows, 32 columns at a time, with
  // all of those loads in flight together (the copy is latency-bound otherwise)
#pragma unroll
  for (int c0 = 0; c0 < SNB; c0 += 32) {
    float t[TRPL][32];
#pragma unroll
    for (int r = 0; r < TRPL; ++r) {
      const int il = tid + TPT * r;
#pragma unroll
      for (int c = 0; c < 32; ++c)
        t[r][c] = (il < nr && c0 + c < jb) ? (float)W[(r0 + il) + (int64_t)(c0 + c) * ldw] : 0.f;
    }
#pragma unroll
    for (int r = 0; r < TRPL; ++r) {
      const int il = tid + TPT * r;
      if (il < nr)
#pragma unroll
        for (int c = 0; c < 32; ++c) sp[(c0 + c) * RP + il] = t[r][c];
    }
  }
  for (int il = tid; il < nr; il += TPT) rstate[il] = -1;  // -1: not a pivot yet; j: the pivot of column j
  if (tid == 0) {
    sm100::mbar_init(&xbar[0], 1);
    sm100::mbar_init(&xbar[1], 1);
    sm100::fence_mbar_init();
    sfail = 0;
  }
  __syncthreads();
  cluster.sync();  // every CTA runs, its mbarriers initialised, before the first push

  bool failed = false;
  uint64_t umax = 0, umin = ~0ull;  // |u_jj| bits (CTA 0, thread 0)
  const int ngroups = (int)cdiv(jb, TG);
  for (int g = 0; g < ngroups; ++g) {
    const int c0 = g * TG, gw = (int)imin(TG, jb - c0), par = g & 1, ub = g & 1;
    const int pb = c0 >= TG ? c0 - TG : 0;  // first pushed column: the previous group's multipliers on
    const int nv = SNB - pb;                // values pushed per nominee (a multiple of 8)
    const int nq = 1 + nv / 4;
    if (tid == 0) sm100::mbar_arrive_expect_tx(&xbar[par], (uint32_t)(C * gw * sizeof(TSlot)));
    // -- 1-2. the CTA's nominees: partial pivoting over all of its rows on
    // the group's columns (scratch copies in registers), every warp taking
    // part in every step
    {
      float v[TRPL][TG];
      bool live[TRPL];
#pragma unroll
      for (int r = 0; r < TRPL; ++r) {
        const int il = tid + TPT * r;
        live[r] = il < nr && rstate[il] < 0;
#pragma unroll
        for (int k = 0; k < TG; ++k) v[r][k] = live[r] ? sp[(c0 + k) * RP + il] : 0.f;
      }
      const int cnt = group_gepp<TRPL, TPT / 32, false>(v, live, gw, selw[0], 1, gwmax, gprow, nullptr, nullptr,
                                                        nullptr, 0);
      if (tid < TG) cand2[tid] = tid < cnt ? selw[0][tid] : -1;
      // the previous group's bulk pushes have read the staging slots
      if (tid < C) sm100::bulk_wait_read0();
    }
    __syncthreads();
    // -- 3. push the nominees (columns pb..63): staged as gw slots, then one
    // bulk copy into every CTA (slots cr * gw .. of its buffer par)
    for (int e = tid; e < gw * nq; e += TPT) {
      const int q = e % nq, s2 = e / nq;
      const int il = cand2[s2];
      if (q == 0) {
        stage[s2].row = il >= 0 ? (uint32_t)(r0 + il) : 0xFFFFFFFFu;
      } else {
        const int k = (q - 1) * 4;
        float4 w4;
        w4.x = il >= 0 ? sp[(pb + k) * RP + il] : 0.f;
        w4.y = il >= 0 ? sp[(pb + k + 1) * RP + il] : 0.f;
        w4.z = il >= 0 ? sp[(pb + k + 2) * RP + il] : 0.f;
        w4.w = il >= 0 ? sp[(pb + k + 3) * RP + il] : 0.f;
        *reinterpret_cast<float4 *>(&stage[s2].v[k]) = w4;
      }
    }
    sm100::fence_proxy_async_smem();  // the staged slots, visible to the bulk copies
    __syncthreads();
    if (tid < C) {  // lane d of warp 0 pushes into CTA d
      bulk_push(sm100::cluster_addr(&slots[(size_t)par * C * TG + cr * gw], tid), stage, (uint32_t)(gw * sizeof(TSlot)),
                sm100::cluster_addr(&xbar[par], tid));
      sm100::bulk_commit();
    }
    // -- 4. the previous group's update on the columns right of this group
    // (a thread's rows and 4 columns at a time: 8 independent chains of the
    // 8 dependent FMAs of rank8 in flight; SNB - c0 - TG is a multiple of 8)
    if (g > 0) {
      const float(*U)[TG] = UgT[ub ^ 1];
      bool on[TRPL];
      float l[TRPL][TG];
#pragma unroll
      for (int r = 0; r < TRPL; ++r) {
        const int il = tid + TPT * r;
        on[r] = il < nr && rstate[il] < 0;
#pragma unroll
        for (int s2 = 0; s2 < TG; ++s2) l[r][s2] = on[r] ? sp[(pb + s2) * RP + il] : 0.f;
      }
      for (int k0 = c0 + TG; k0 < SNB; k0 += 4) {
        float x[TRPL][4];
#pragma unroll
        for (int r = 0; r < TRPL; ++r)
#pragma unroll
          for (int j = 0; j < 4; ++j) x[r][j] = on[r] ? sp[(k0 + j) * RP + tid + TPT * r] : 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float4 u0 = *reinterpret_cast<const float4 *>(&U[k0 + j][0]);
          const float4 u1 = *reinterpret_cast<const float4 *>(&U[k0 + j][4]);
#pragma unroll
          for (int r = 0; r < TRPL; ++r) x[r][j] = rank8(x[r][j], l[r], u0, u1);
        }
#pragma unroll
        for (int r = 0; r < TRPL; ++r)
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (on[r]) sp[(k0 + j) * RP + tid + TPT * r] = x[r][j];
      }
    }
    // every CTA's nominees have landed (bounded: a missing push sets the
    // error flag and ends the panel, never a hang)
    if (!sm100::bounded_wait(&xbar[par], (uint32_t)(g >> 1) & 1u)) sfail = 1;
    __syncthreads();
    if (sfail) {
      if (tid == 0) atomicExch(err, 5);
      failed = true;
      break;
    }
    const TSlot *sl = slots + (size_t)par * C * TG;
    // -- 5. the group's pivots from all nominees, the same in every CTA
    // (warps 0-3, one candidate per lane)
    if (warp < 4) {
      float v[1][TG];
      bool live[1];
      live[0] = tid < C * gw && sl[tid].row != 0xFFFFFFFFu;
#pragma unroll
      for (int k = 0; k < TG; ++k) v[0][k] = live[0] ? sl[tid].v[c0 - pb + k] : 0.f;
      const int cnt = group_gepp<1, 4, true>(v, live, gw, selw[1], 2, gwmax, gprow, Lsm, Lg, &UgT[ub][c0][0], TG);
      if (warp == 0) {
        // the panel always has at least gw rows that are not pivots yet, so
        // cnt == gw; a shortfall would mean a corrupted exchange
        if (cnt < gw && lane == 0) atomicExch(err, 6);
        if (lane < gw) {
          const int s2 = selw[1][lane];
          wslot[lane] = lane < cnt ? s2 : -1;
          win[c0 + lane] = lane < cnt ? (int32_t)sl[s2].row : -1;
        }
        // the inverse of the group's unit-lower block of L: lane q forms column q
        __syncwarp();
        if (lane < TG) {
          float col[TG];
#pragma unroll
          for (int t = 0; t < TG; ++t) {
            float x = t == lane ? 1.f : 0.f;
#pragma unroll
            for (int p = 0; p < t; ++p) x = fmaf(-Lg[t][p], col[p], x);
            col[t] = t < lane ? 0.f : x;
          }
#pragma unroll
          for (int t = 0; t < TG; ++t) Linv[t][lane] = col[t];
        }
      }
    } else if (!SEL && cr == 0 && tid == TPT / 2) {
      // meanwhile (warps 4-7 are idle): LAPACK's interchanges for the
      // previous group's pivots
      if (g == 0) interchanges_init(jb, posin, at_);
      for (int j = c0 - TG; j >= 0 && j < c0; ++j) ipiv[j] = interchange_step(j, win[j], jb, col0, posin, at_);
    }
    __syncthreads();
    if (win[c0 + gw - 1] < 0) {  // (err is set) leave the group loop uniformly
      failed = true;
      break;
    }
    // the pivots' pushed rows, brought up to date on the columns right of the
    // group with the previous group's update (their multipliers of that group
    // are the first 8 pushed values), in place
    if (g > 0) {
      TSlot *slw = slots + (size_t)par * C * TG;
      const float(*U)[TG] = UgT[ub ^ 1];
      const int nk = SNB - c0 - gw;
      for (int e = tid; e < gw * nk; e += TPT) {
        const int ci = wslot[e / nk], k = c0 + gw + e % nk;
        float l[TG];
#pragma unroll
        for (int s2 = 0; s2 < TG; ++s2) l[s2] = slw[ci].v[s2];
        slw[ci].v[k - pb] = rank8(slw[ci].v[k - pb], l, *reinterpret_cast<const float4 *>(&U[k][0]),
                                  *reinterpret_cast<const float4 *>(&U[k][4]));
      }
      __syncthreads();
    }
    // the pivots' U rows right of the group: U = Linv A' over the up-to-date
    // pushed rows A', one (row, column) element per thread
    for (int e = tid; e < gw * (SNB - c0 - gw); e += TPT) {
      const int t = e % gw, k = c0 + gw + e / gw;
      float u = 0.f;
#pragma unroll
      for (int q = 0; q < TG; ++q)
        if (q <= t) u = fmaf(Linv[t][q], sl[wslot[q]].v[k - pb], u);
      UgT[ub][k][t] = u;
    }
    if (tid < gw) {
      const float pv = UgT[ub][c0 + tid][tid];
      invp[tid] = pv != 0.f ? __frcp_rn(pv) : 0.f;
      const int row = win[c0 + tid];
      if (row >= r0 && row < r1) rstate[row - r0] = (int16_t)(c0 + tid);
    }
    if (cr == 0 && tid == TPT - 1) {
      for (int t = 0; t < gw; ++t) {
        const float pv = UgT[ub][c0 + t][t];
        if (!SEL && pv == 0.f) atomicCAS(info, 0, col0 + c0 + t + 1);
        const uint64_t ab = __float_as_uint(pv) & 0x7fffffffu;
        if (ab <= 0x7f800000u) {
          umax = ab > umax ? ab : umax;
          umin = ab < umin ? ab : umin;
        }
      }
    }
    __syncthreads();
    // -- 6. this CTA's pivot rows take their final values (all threads, an
    // element each); the other rows their multipliers and the update of the
    // next group's columns
    for (int e = tid; e < gw * (SNB - c0); e += TPT) {
      const int t = e / (SNB - c0), k = c0 + e % (SNB - c0);
      const int row = win[c0 + t];
      if (row < r0 || row >= r1) continue;
      sp[k * RP + (row - r0)] = k < c0 + t ? Lg[t][k - c0] : UgT[ub][k][t];
    }
    // (a thread's rows side by side, so that their dependent chains overlap;
    // pivot rows, of this group or earlier, are left as they are)
    {
      bool on[TRPL];
      float l[TRPL][TG];
#pragma unroll
      for (int r = 0; r < TRPL; ++r) {
        const int il = tid + TPT * r;
        on[r] = il < nr && rstate[il] < 0;
      }
#pragma unroll
      for (int s2 = 0; s2 < TG; ++s2) {
#pragma unroll
        for (int r = 0; r < TRPL; ++r) {
          const int il = tid + TPT * r;
          const bool live = on[r] && s2 < gw;
          float a = live ? sp[(c0 + s2) * RP + il] : 0.f;
#pragma unroll
          for (int q = 0; q < s2; ++q) a = fmaf(-l[r][q], UgT[ub][c0 + s2][q], a);
          l[r][s2] = live ? a * invp[s2] : 0.f;
          if (live) sp[(c0 + s2) * RP + il] = l[r][s2];
        }
      }
      if (c0 + TG < SNB) {  // the next group's 8 columns
#pragma unroll
        for (int j = 0; j < TG; ++j) {
          const int k = c0 + TG + j;
          const float4 u0 = *reinterpret_cast<const float4 *>(&UgT[ub][k][0]);
          const float4 u1 = *reinterpret_cast<const float4 *>(&UgT[ub][k][4]);
#pragma unroll
          for (int r = 0; r < TRPL; ++r) {
            const int il = tid + TPT * r;
            if (on[r]) sp[k * RP + il] = rank8(sp[k * RP + il], l[r], u0, u1);
          }
        }
      }
    }
    __syncthreads();
  }
  if (!failed) {
    if constexpr (SEL) {
      if (cr == 0)
        for (int t = tid; t < jb; t += TPT) winout[t] = win[t];
      // the pivot rows' FP64 values, each CTA its own rows
      for (int e = tid; e < jb * jb; e += TPT) {
        const int t = e / jb, c = e % jb, row = win[t];
        if (row >= r0 && row < r1) sel[t * SNB + c] = W[row + (int64_t)c * ldw];
      }
    } else {
    // -- the last group's interchanges (CTA 0; the earlier groups' ran
    // during the searches that followed them)
    if (cr == 0 && tid == TPT / 2)
      for (int j = (ngroups - 1) * TG; j < jb; ++j) ipiv[j] = interchange_step(j, win[j], jb, col0, posin, at_);
    if (track != nullptr && cr == 0 && tid == TPT - 1) {
      if (umin != ~0ull) {
        const uint64_t mx = (uint64_t)__double_as_longlong((double)__uint_as_float((uint32_t)umax));
        const uint64_t mn = (uint64_t)__double_as_longlong((double)__uint_as_float((uint32_t)umin));
        if (mx > track[0]) track[0] = mx;
        if (mn < track[1]) track[1] = mn;
      }
      const double gmx = __longlong_as_double((long long)track[0]), gmn = __longlong_as_double((long long)track[1]);
      const double spread = gmn > 0.0 ? gmx / gmn : INFINITY;
      if (give_up_now(spread, give_up, col0 + jb, col0 + mp)) *(volatile int32_t *)(track + 2) = 1;
    }
    __syncthreads();
    // -- write back the panel: first every row where it started, as float4
    // runs of 4 rows (a warp writes 512 contiguous bytes of a column; R is a
    // multiple of 4, so runs start 16-byte aligned in W when W and ldw allow);
    // the rows that move (the pivots, and CTA 0's first jb rows that are not
    // pivots) are written again to their final positions after the cluster
    // barrier below, so that those writes land last
    const bool vec = (ldw & 3) == 0 && (reinterpret_cast<uintptr_t>(W) & 15) == 0 && (R & 3) == 0;
    if (vec) {
      const int nq4 = nr / 4;
      for (int e = tid; e < nq4 * jb; e += TPT) {
        const int il0 = 4 * (e % nq4), c = e / nq4;
        *reinterpret_cast<float4 *>(&W[(r0 + il0) + (int64_t)c * ldw]) =
            *reinterpret_cast<const float4 *>(&sp[c * RP + il0]);
      }
      for (int e = tid; e < (nr - 4 * nq4) * jb; e += TPT) {
        const int il = 4 * nq4 + e % (nr - 4 * nq4), c = e / (nr - 4 * nq4);
        W[(r0 + il) + (int64_t)c * ldw] = sp[c * RP + il];
      }
    } else {
#pragma unroll
      for (int r = 0; r < TRPL; ++r) {
        const int il = tid + TPT * r;
        if (il >= nr) continue;
#pragma unroll 8
        for (int c = 0; c < jb; ++c) W[(r0 + il) + (int64_t)c * ldw] = sp[c * RP + il];
      }
    }
    if (plan != nullptr && cr == 0 && warp == 0) list_panel_moves(win, posin, jb, col0, plan);
    }
  }
  if (tid < C) sm100::bulk_wait_read0();  // this CTA's last pushes have read its staging slots
  cluster.sync();  // no CTA leaves while another may still push into it
  if constexpr (!SEL) {
    if (!failed) {
      // the rows that move, over their first write: the pivot of column t
      // (panel row win[t]) to position t, lanes on consecutive t; CTA 0's
      // first jb rows that are not pivots to where the interchanges put them
      for (int e = tid; e < jb * jb; e += TPT) {
        const int t = e % jb, c = e / jb, x = win[t];
        if (x >= r0 && x < r1) W[t + (int64_t)c * ldw] = sp[c * RP + (x - r0)];
      }
      if (cr == 0)
        for (int e = tid; e < jb * jb; e += TPT) {
          const int il = e % jb, c = e / jb;
          if (rstate[il] < 0) W[posin[il] + (int64_t)c * ldw] = sp[c * RP + il];
        }
    }
  }
}

template <typename G>
int launch_tpanel(cudaStream_t s, G *W, int64_t ldw, int64_t mp, int jb, int32_t *ipiv, int32_t col0,
                  int32_t *info, int32_t *plan, uint64_t *track, double give_up, int32_t *err,
                  int32_t *winout = nullptr, G *sel = nullptr) {
  const int C = (int)imin(SMAXC, imax(1, cdiv(mp, TPT)));
  // rows per CTA, a multiple of 4 (the write-back's float4 runs); C <= 16
  // keeps the last CTA's share positive: mp > 256 (C - 1) > 4 C (C - 1)
  const int64_t R = cdiv(cdiv(mp, C), 4) * 4;
  // CTA 0 must hold the panel's first jb rows (the interchange bookkeeping)
  if (R > (int64_t)TPT * TRPL || R < jb)
    return fail(BOLA_ERR_UNSUPPORTED, "mixed LU: panel of %lld x %d not supported", (long long)mp, jb);
  const size_t smem = tpanel_smem(R, C);
  static bool attr = false;
  if (!attr) {
    BOLA_TRY_CUDA(cudaFuncSetAttribute(tpanel_kernel<G>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    BOLA_TRY_CUDA(cudaFuncSetAttribute(tpanel_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)tpanel_smem(TPT * TRPL, SMAXC)));
    attr = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C, 1, 1);
  cfg.blockDim = dim3(TPT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[2];  // the cluster; a programmatic dependent of the previous step's kernel
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  ProfScope prof(s, std::is_same<G, double>::value ? "tselect64" : "tpanel", (double)mp * jb * jb,
                 8.0 * (double)mp * jb);
  BOLA_TRY_CUDA(cudaLaunchKernelEx(&cfg, tpanel_kernel<G>, W, ldw, mp, jb, ipiv, col0, info, R, plan, track,
                                   give_up, err, winout, sel));
  return 0;
}

// ---- the FP64-accurate factor's panel ------------------------------------------
// Column-by-column partial pivoting in FP64 costs, per column, a cluster
// exchange, four CTA barriers and the column's FP64 update confined to the
// panel's CTAs.  The FP64-storage factor splits its panel instead, as
// communication-avoiding LU (CALU) does:
//   1. tpanel_kernel<double> chooses the jb pivot rows by tournament on FP32
//      copies of the panel (W's column blocks are scaled to O(1), and FP32
//      is ample for choosing pivots);
//   2. panel_lu64 factors the panel in FP64 in the tournament's pivot order
//      without further pivoting (CALU's final step): the selected block and
//      the rows below it, on one CTA per 64 rows, each factoring the block
//      itself; it derives LAPACK's interchanges, puts the rows they displace
//      below the block, tracks the pivots and writes the update's operand
//      (exact bf16 slices of each row of L21).

// 1 / p for the FP64 panel's pivots without the long-latency division:
// Newton's iteration for the reciprocal, r <- r (2 - p r), from the FP32
// reciprocal as its seed (relative error 2^-23 -> 2^-46 -> below 2^-52 after
// two steps); plain division where |p| lies outside [2^-100, 2^101), so that
// the FP32 seed is a normal number.
__device__ __forceinline__ double recip64(double p) {
  const int e = (int)(((uint64_t)__double_as_longlong(p) >> 52) & 0x7FF);  // biased exponent (integer pipe)
  if (e < 1023 - 100 || e > 1023 + 100) return 1.0 / p;
  double r = (double)__frcp_rn((float)p);
  r = r * fma(-p, r, 2.0);
  r = r * fma(-p, r, 2.0);
  return r;
}

// Steps 2 and 3 of the panel above in one launch (Wp: the panel's top-left,
// rows col0.. of W).  The tournament has fixed the pivot order (row win[q]
// is the pivot of column q, chosen by partial pivoting among the nominees),
// so the panel is factored without further pivoting, as CALU's last step
// does: the selected block and every row below it go through the same 64
// right-looking steps.  CTA i < nA takes the panel's rows at positions
// 64 (i + 1) .. 64 (i + 1) + 63 that are not pivots (they stay where they
// are); the last CTA takes the first 64 rows that are not pivots (they move
// to the pivots' old positions).  (128 rows a CTA, on half the SMs, measured
// slower: each CTA's FP64 pipe bounds it.)  Every CTA factors the 64 x 64
// block itself, with the same arithmetic (so the same U11 everywhere), from
// the copy of the pivot rows that the selection made (sel): no CTA reads a
// part of W that another one writes.  Rows in shared memory, four lanes per row, lane h
// updating columns c = h (mod 4), so every FP64 warp instruction has 32 busy
// lanes; warps 0-7 hold the block (a warp whose rows are done stops
// issuing), warps 8-15 the rows below, warp 16 forms the next pivot's
// reciprocal behind a named barrier while the rows update.  On GB300 a
// warp's other instructions wait while its FP64 instruction is dispatched
// (~64 cycles), so several warps share each sub-partition.  Per column k (a
// rolled loop: an unrolled one misses the instruction cache): every row's
// multiplier, its column k + 1 first, then its other columns.  The last CTA
// also derives LAPACK's interchanges (on warp 0 once its block rows are
// done), the swap plan, the block and the pivots' spread; every CTA writes
// its rows' L21 and their exact bf16 slices (the update's A operand).
constexpr int PL_LPR = 4;                          // lanes per row
constexpr int PL_SLOTS = SNB;                      // rows below the block per CTA
constexpr int PL_ROWS = SNB + PL_SLOTS;            // block rows + rows below
constexpr int PL_RWARPS = PL_ROWS * PL_LPR / 32;   // 16 warps with rows
constexpr int PL_BWARPS = SNB * PL_LPR / 32;       // 8 of them the block's
constexpr int PL_THREADS = PL_RWARPS * 32 + 32;    // and the reciprocal warp: 544
constexpr size_t PL_SMEM = sizeof(double) * PL_ROWS * (SNB + 1);
__global__ void __launch_bounds__(PL_THREADS, 1)
panel_lu64(double *Wp, int64_t ldw, int64_t mp, int jb, int32_t col0, const int32_t *win_in, const double *sel,
           int32_t *plan, int32_t *ipiv, int32_t *info, uint64_t *track, double give_up, int32_t *err, void *aop,
           int32_t *aexp, int64_t cap) {
  sm100::grid_dependency_wait();
  const int nA = (int)gridDim.x - 1;
  const bool top = (int)blockIdx.x == nA;
  // an abandoned factorisation (flag set by an earlier panel on this stream):
  // identity pivots keep ipiv valid for the kernels that compose it
  if (track != nullptr && *(volatile const int32_t *)(track + 2) != 0) {
    if (top)
      for (int t = threadIdx.x; t < jb; t += blockDim.x) ipiv[t] = col0 + t + 1;
    return;
  }
  extern __shared__ __align__(16) double pl_raw[];
  double(*a)[SNB + 1] = reinterpret_cast<double(*)[SNB + 1]>(pl_raw);  // rows 0..63: the block; 64 + i: slot i
  __shared__ int32_t win[SNB], pivl[SNB], posin[SNB], at_[SNB], rows_s[2 * SNB], src_s[2 * SNB];
  __shared__ int32_t slot[PL_SLOTS];  // panel position of slot i's row (-1: none)
  __shared__ double rinv_s[2];   // 1 / the pivot of column k (k & 1)
  __shared__ int bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = tid / PL_LPR, h = tid % PL_LPR;
  const int64_t base = top ? 0 : PL_SLOTS + (int64_t)blockIdx.x * PL_SLOTS;  // panel position of slot 0
  if (tid == 0) bad = 0;
  if (tid < PL_SLOTS) slot[tid] = 0;
  __syncthreads();
  for (int t = tid; t < jb; t += PL_THREADS) {
    const int w = win_in[t];
    win[t] = w;
    // a selection that did not finish (its exchange gave up and set the
    // error word) leaves no valid list: stop here rather than index W with it
    if (w < 0 || w >= mp) atomicExch(&bad, 1);
    else if (w >= base && w < base + PL_SLOTS) slot[w - base] = -1;  // a pivot: not one of this CTA's rows
  }
  __syncthreads();
  if (bad != 0) {
    if (top) {
      if (tid == 0) atomicExch(err, 7);
      for (int t = tid; t < jb; t += PL_THREADS) ipiv[t] = col0 + t + 1;
    }
    return;
  }
  if (tid < PL_SLOTS) {
    const int64_t p = base + tid;
    slot[tid] = (slot[tid] == 0 && p < mp) ? (int32_t)p : -1;
  }
  __syncthreads();
  // the block (from sel) and this CTA's rows (from W), all of a thread's
  // loads in flight together
  if (tid < PL_RWARPS * 32) {
    constexpr int PER = PL_ROWS * SNB / (PL_RWARPS * 32);  // 16
    double v[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = tid + PL_RWARPS * 32 * u;
      if (e < SNB * SNB) {
        const int r = e / SNB, c = e % SNB;
        v[u] = (r < jb && c < jb) ? sel[r * SNB + c] : 0.0;
      } else {
        const int r = (e - SNB * SNB) % PL_SLOTS, c = (e - SNB * SNB) / PL_SLOTS;
        const int s2 = slot[r];
        v[u] = (s2 >= 0 && c < jb) ? Wp[s2 + (int64_t)c * ldw] : 0.0;
      }
    }
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = tid + PL_RWARPS * 32 * u;
      if (e < SNB * SNB)
        a[e / SNB][e % SNB] = v[u];
      else
        a[SNB + (e - SNB * SNB) % PL_SLOTS][(e - SNB * SNB) / PL_SLOTS] = v[u];
    }
  }
  uint64_t umax = 0, umin = ~0ull;  // |u_kk| bits (the reciprocal warp's lane 0)
  // 1 / the pivot of column k into rinv_s[k & 1], with the pivots' extent and
  // the first zero pivot
  auto pivot = [&](double pv, int k) {
    const uint64_t ab = (uint64_t)__double_as_longlong(pv) & 0x7fffffffffffffffull;
    rinv_s[k & 1] = ab != 0 ? recip64(pv) : 0.0;
    if (ab == 0 && top) atomicCAS(info, 0, col0 + k + 1);
    if (ab <= 0x7ff0000000000000ull) {
      umax = ab > umax ? ab : umax;
      umin = ab < umin ? ab : umin;
    }
  };
  const bool rwarp = warp == PL_RWARPS;  // the reciprocal warp (no rows)
  if (top && tid == 0) interchanges_init(jb, posin, at_);
  __syncthreads();
  if (rwarp && lane == 0) pivot(a[0][0], 0);
  int jdone = 0;  // (thread 0 of the last CTA) columns whose interchange is done
#pragma unroll 1
  for (int k = 0; k < jb; ++k) {
    const int hk = k % PL_LPR;
    // column k's pivot row and reciprocal are final
    asm volatile("bar.sync 1, %0;" ::"r"(PL_THREADS) : "memory");
    if (rwarp) {
      // the next pivot, once its row's warp has updated it (named barrier 2:
      // that warp arrives, this one waits), while the rows' other columns are
      // updated; the dependent FP64 chain of the reciprocal stays off the
      // row warps
      if (k + 1 < jb) {
        asm volatile("bar.sync 2, 64;" ::: "memory");
        if (lane == 0) pivot(a[k + 1][k + 1], k + 1);
      }
      continue;
    }
    if (warp < PL_BWARPS && (warp + 1) * (32 / PL_LPR) - 1 <= k) {  // every block row of this warp is done
      // warp 0, idle from column 7 on, runs LAPACK's interchanges for the
      // pivots, two per column until it has caught up
      if (top && tid == 0)
        for (int u = 0; u < 2 && jdone <= k; ++u, ++jdone) {
          pivl[jdone] = win[jdone];
          ipiv[jdone] = interchange_step(jdone, win[jdone], jb, col0, posin, at_);
        }
      continue;
    }
    const bool act = q >= SNB || (q > k && q < jb);  // (rows below: every step; an empty slot holds zeros)
    const double l = act ? a[q][k] * rinv_s[k & 1] : 0.0;
    __syncwarp();  // the quad has read a[q][k] before it becomes the multiplier
    if (act) {
      if (h == hk) a[q][k] = l;
      // column k + 1 first: the next pivot
      if (k + 1 < jb && h == (k + 1) % PL_LPR) a[q][k + 1] = fma(-l, a[k][k + 1], a[q][k + 1]);
    }
    if (k + 1 < jb && warp == (k + 1) / (32 / PL_LPR)) {  // the next pivot's warp hands it over
      __threadfence_block();
      __syncwarp();
      asm volatile("bar.arrive 2, 64;" ::: "memory");
    }
    // the row's other columns c = 4u + h >= k + 2: the same trip count in
    // every lane of the warp (a per-lane start would split the warp into
    // paths that each dispatch their own FP64 instructions), 4 columns at a
    // time with all of their loads issued before the FMAs
    for (int u0 = (k + 2) / PL_LPR; u0 < SNB / PL_LPR; u0 += 4) {
      double pr[4], xr[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = PL_LPR * (u0 + u) + h;
        const bool on = act && u0 + u < SNB / PL_LPR && c >= k + 2 && c < jb;
        pr[u] = on ? a[k][c] : 0.0;
        xr[u] = on ? a[q][c] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = PL_LPR * (u0 + u) + h;
        if (act && u0 + u < SNB / PL_LPR && c >= k + 2 && c < jb) a[q][c] = fma(-l, pr[u], xr[u]);
      }
    }
  }
  if (top && tid == 0)  // the interchanges still to run (the last columns, or all of a narrow block)
    for (; jdone < jb; ++jdone) {
      pivl[jdone] = win[jdone];
      ipiv[jdone] = interchange_step(jdone, win[jdone], jb, col0, posin, at_);
    }
  __syncthreads();
  if (top && warp == 0) list_panel_moves(pivl, posin, jb, col0, plan, rows_s, src_s);
  // -- this CTA's rows: L21 to their final positions (the last CTA's to
  // where the interchanges put them) and their exact bf16 slices, one
  // exponent per row
  if (q >= SNB && warp < PL_RWARPS) {
    const int i = q - SNB, s2 = slot[i];
    double x[SNB / PL_LPR];
    uint64_t mb = 0;
#pragma unroll
    for (int u = 0; u < SNB / PL_LPR; ++u) {
      x[u] = a[q][PL_LPR * u + h];
      const uint64_t m = oz_mag(x[u]);
      mb = m > mb ? m : mb;
    }
#pragma unroll
    for (int off = 1; off < PL_LPR; off <<= 1) {  // the row's other lanes
      const uint64_t om = __shfl_xor_sync(0xffffffffu, mb, off);
      mb = om > mb ? om : mb;
    }
    if (s2 >= 0) {
      const int64_t fp = s2 < jb ? posin[s2] : s2;  // (only the last CTA has rows among the first jb)
#pragma unroll
      for (int u = 0; u < SNB / PL_LPR; ++u) {
        const int c = PL_LPR * u + h;
        if (c < jb) Wp[fp + (int64_t)c * ldw] = x[u];
      }
      if (aop != nullptr) {
        const int e = oz_exponent(mb);
        const int64_t orow = fp - jb;
        if (h == 0) aexp[orow] = e;
        __nv_bfloat16 *out = static_cast<__nv_bfloat16 *>(aop);
#pragma unroll
        for (int u = 0; u < SNB / PL_LPR; ++u) {
          __nv_bfloat16 sl[OZ_SLICES];
          oz_slices(x[u], e, sl);
#pragma unroll
          for (int t = 0; t < OZ_SLICES; ++t) out[((int64_t)t * cap + orow) * SNB + PL_LPR * u + h] = sl[t];
        }
      }
    }
  }
  if (top) {
    // the factored block (unit-lower L11 below the diagonal, U11 on and above)
    for (int e = tid; e < jb * jb; e += PL_THREADS) {
      const int r = e % jb, c = e / jb;
      Wp[r + (int64_t)c * ldw] = a[r][c];
    }
    if (track != nullptr && rwarp && lane == 0) {
      // the running extent of |u_ii| and the give-up test
      if (umin != ~0ull) {
        if (umax > track[0]) track[0] = umax;
        if (umin < track[1]) track[1] = umin;
      }
      const double gmx = __longlong_as_double((long long)track[0]), gmn = __longlong_as_double((long long)track[1]);
      const double spread = gmn > 0.0 ? gmx / gmn : INFINITY;
      if (give_up_now(spread, give_up, col0 + jb, col0 + mp)) *(volatile int32_t *)(track + 2) = 1;
    }
  }
}

// Rows r0 .. r0 + 63 of the update's K-major A operand (kinds 0-2) from the
// factored panel: operand row r is row j + 64 + r of W's columns j .. j + 63
// (final once the panel kernel has written them back), rounded as
// write_operand_row rounds.  The 64 x 64 tile is read a column at a time and
// written a row at a time, both coalesced, through t (64 x 64, columns
// XOR-swizzled by the row so that both passes are free of bank conflicts).
__device__ __forceinline__ void operand_tile(const float *W, int64_t ldw, int64_t j, int64_t m2, int64_t r0,
                                             int kind, void *op, float *op_lo, float *t) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rows = (int)imin(SNB, m2 - r0);
  const float *src = W + (j + SNB + r0) + j * ldw;
  constexpr int PER = SNB * SNB / 256;
  float v[PER];
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = tid + 256 * q, r = e % SNB, c = e / SNB;
    v[q] = r < rows ? src[r + (int64_t)c * ldw] : 0.f;
  }
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = tid + 256 * q, r = e % SNB, c = e / SNB;
    t[r * SNB + (c ^ (r & 31))] = v[q];
  }
  __syncthreads();
  for (int r = warp; r < rows; r += 8) {
    const float a = t[r * SNB + (lane ^ (r & 31))], b = t[r * SNB + ((lane + 32) ^ (r & 31))];
    const int64_t orow = r0 + r;
    if (kind == 0) {
      __nv_bfloat16 *d = static_cast<__nv_bfloat16 *>(op) + orow * SNB;
      d[lane] = __float2bfloat16_rn(a);
      d[lane + 32] = __float2bfloat16_rn(b);
    } else {
      float *d = static_cast<float *>(op) + orow * SNB;
      const float ha = tf32_round(a), hb = tf32_round(b);
      d[lane] = ha;
      d[lane + 32] = hb;
      if (kind == 2) {
        float *dl = op_lo + orow * SNB;
        dl[lane] = tf32_round(a - ha);
        dl[lane + 32] = tf32_round(b - hb);
      }
    }
  }
}

// The panel's interchanges on the columns right of it, U12 = L11^-1 A12 and
// its K-major B operand: a warp per column, ncta CTAs (the finished columns
// left of the panel take the interchanges once, when the factorisation is
// done: apply_left_swaps).  CTA 0 also applies them to the row permutation.
// The FP32 factors' CTAs from ncta on write the A operand of the update (aop:
// operand_tile, one 64-row tile each).
template <typename T>
__global__ void __launch_bounds__(256)
sswap_trsm(T *W, int64_t ldw, int64_t n, int64_t j, int jb, const int32_t *plan, int kind, void *bop,
           float *bop_lo, int32_t *bexp, int64_t cap, const int32_t *abort, int ncta, void *aop, float *aop_lo,
           int32_t *perm) {
  sm100::grid_dependency_wait();
  if (abort != nullptr && *(volatile const int32_t *)abort != 0) return;  // set before this launch (same stream)
  __shared__ int32_t rows[2 * SNB], src[2 * SNB];
  __shared__ __align__(16) T L[SNB * SNB];
  __shared__ int cnt;
  if constexpr (std::is_same<T, float>::value) {
    if ((int)blockIdx.x >= ncta) {
      operand_tile(W, ldw, j, n - j - jb, (int64_t)((int)blockIdx.x - ncta) * SNB, kind, aop, aop_lo, L);
      return;
    }
  }
  // the interchanges, composed once by the panel kernel
  if (threadIdx.x == 0) cnt = plan[0];
  for (int t = threadIdx.x; t < 2 * SNB; t += blockDim.x) {
    rows[t] = plan[1 + t];
    src[t] = plan[1 + 2 * SNB + t];
  }
  // the 64 x 64 diagonal block (L11 below its diagonal), all of a thread's loads in flight together
  {
    constexpr int PER = SNB * SNB / 256;
    T t[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int e = threadIdx.x + 256 * q;
      const int r = e % SNB, c = e / SNB;
      t[q] = (r < jb && c < jb) ? W[(j + r) + (j + c) * ldw] : T(0);
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) L[threadIdx.x + 256 * q] = t[q];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  if (perm != nullptr && blockIdx.x == 0 && threadIdx.x < 32) {
    // the same moves on the row permutation (warp 0 of CTA 0, besides its column)
    int32_t pv[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) pv[e] = lane + 32 * e < cnt ? perm[src[lane + 32 * e]] : 0;
    __syncwarp();
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (lane + 32 * e < cnt) perm[rows[lane + 32 * e]] = pv[e];
  }
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= n - j - jb) return;
  const int64_t col = j + jb + w;
  T *cp = W + col * ldw;
  T v[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) v[e] = lane + 32 * e < cnt ? cp[src[lane + 32 * e]] : T(0);
  __syncwarp();
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (lane + 32 * e < cnt) cp[rows[lane + 32 * e]] = v[e];
  __syncwarp();
  T b0 = lane < jb ? cp[j + lane] : T(0);
  T b1 = lane + 32 < jb ? cp[j + lane + 32] : T(0);
  // rows 0..31 take updates from k < 32 only: two loops, so that no warp
  // instruction runs with every lane idle (an FP64 one costs its full slot)
  const int k0 = jb < 32 ? jb : 32;
  for (int k = 0; k < k0; ++k) {
    const T bk = __shfl_sync(0xffffffffu, b0, k);
    if (lane > k) b0 = fmaT(-L[lane + k * SNB], bk, b0);
    if (lane + 32 < jb) b1 = fmaT(-L[lane + 32 + k * SNB], bk, b1);
  }
  for (int k = 32; k < jb; ++k) {
    const T bk = __shfl_sync(0xffffffffu, b1, k - 32);
    if (lane + 32 > k && lane + 32 < jb) b1 = fmaT(-L[lane + 32 + k * SNB], bk, b1);
  }
  if (lane < jb) cp[j + lane] = b0;
  if (lane + 32 < jb) cp[j + lane + 32] = b1;
  if (bop != nullptr) {
    // row (col - j - jb) of the K-major B operand: the 64 values of U12's column
    if constexpr (std::is_same<T, float>::value) {
      __shared__ float stage[8][SNB];
      float *st = stage[threadIdx.x >> 5];
      st[lane] = lane < jb ? b0 : 0.f;
      st[lane + 32] = lane + 32 < jb ? b1 : 0.f;
      __syncwarp();
      if (lane == 0) write_operand_row(kind, bop, bop_lo, col - j - jb, st);
    } else {
      oz_split_pair(lane < jb ? (double)b0 : 0.0, lane + 32 < jb ? (double)b1 : 0.0, lane, col - j - jb, cap,
                    static_cast<__nv_bfloat16 *>(bop), bexp);
    }
  }
}

// Once the factorisation is done: every panel's interchanges on the columns
// left of it (the finished L), deferred from the swap kernel.  CTA k takes
// column block k: the moves of panels k+1.. (plans[k'], as the swap kernel
// took them) composed in shared memory into one gather — arr[i] = the
// position, relative to the first row below the block, that the row ending
// in position i held after panel k — then each column's rows below the block
// are read once and the moved ones written back.
template <typename T>
__global__ void __launch_bounds__(512)
apply_left_swaps(T *W, int64_t ldw, int64_t n, const int32_t *plans, const int32_t *abort) {
  if (abort != nullptr && *(volatile const int32_t *)abort != 0) return;
  extern __shared__ __align__(16) unsigned char als_raw[];
  constexpr int NT = 512, U = 16;
  const int k = blockIdx.x, K = (int)cdiv(n, SNB);
  const int64_t base = (int64_t)(k + 1) * SNB;
  const int m = (int)(n - base);
  int32_t *arr = reinterpret_cast<int32_t *>(als_raw);
  T *col = reinterpret_cast<T *>(als_raw + ((sizeof(int32_t) * (size_t)m + 15) & ~(size_t)15));
  for (int i = threadIdx.x; i < m; i += NT) arr[i] = i;
  __syncthreads();
  for (int kp = k + 1; kp < K; ++kp) {
    const int32_t *pl = plans + (int64_t)kp * PLAN_STRIDE;
    const int cnt = pl[0];
    int v = 0, dst = -1;
    if ((int)threadIdx.x < cnt) {
      v = arr[pl[1 + 2 * SNB + threadIdx.x] - base];
      dst = (int)(pl[1 + threadIdx.x] - base);
    }
    __syncthreads();
    if (dst >= 0) arr[dst] = v;
    __syncthreads();
  }
  for (int c = k * SNB; c < (k + 1) * SNB && c < n; ++c) {
    T *cp = W + base + (int64_t)c * ldw;
    for (int i0 = 0; i0 < m; i0 += NT * U) {  // a thread's loads in flight together
      T r[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + (int)threadIdx.x + NT * u;
        r[u] = i < m ? cp[i] : T(0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + (int)threadIdx.x + NT * u;
        if (i < m) col[i] = r[u];
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += NT) {
      const int sidx = arr[i];
      if (sidx != i) cp[i] = col[sidx];
    }
    __syncthreads();
  }
}

__global__ void zero_i32(int32_t *p) { *p = 0; }
__global__ void iota32(int64_t n, int32_t *p) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = (int32_t)i;
}
__global__ void track_init(uint64_t *t) {
  t[0] = 0;                       // max |u_ii| = +0
  t[1] = 0x7ff0000000000000ull;   // min |u_ii| = +inf
  t[2] = 0;                       // not abandoned
}

}  // namespace

int MixedLU::reserve(int64_t n_, int kind_, cudaStream_t s) {
  if (!sp) {
    int least = 0, greatest = 0;
    BOLA_TRY_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    BOLA_TRY_CUDA(cudaStreamCreateWithPriority(&sp, cudaStreamNonBlocking, greatest));
    BOLA_TRY_CUDA(cudaStreamCreateWithPriority(&su, cudaStreamNonBlocking, least));
    for (cudaEvent_t *e : {&ev_in, &ev_sw, &ev_wide, &ev_done})
      BOLA_TRY_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  if (n_ <= cap_n && kind_ == kind && aop[0]) {
    n = n_;
    return 0;
  }
  release(s);
  n = cap_n = n_;
  kind = kind_;
  BOLA_TRY_CUDA(cudaMallocAsync(&err, sizeof(int32_t), s));
  BOLA_TRY_CUDA(cudaMallocAsync(&plan, sizeof(int32_t) * ((size_t)PLAN_STRIDE * cdiv(n, SNB) + SNB), s));
  BOLA_TRY_CUDA(cudaMallocAsync(&track, 4 * sizeof(uint64_t), s));
  BOLA_TRY_CUDA(cudaMemsetAsync(err, 0, sizeof(int32_t), s));
  if (kind == 3) {
    // exact bf16 slices of L21 and U12^T (OZ_SLICES planes of n rows) and their row exponents
    for (int b = 0; b < 2; ++b) {
      BOLA_TRY_CUDA(cudaMallocAsync(&aop[b], (size_t)OZ_SLICES * n * SNB * 2, s));
      BOLA_TRY_CUDA(cudaMallocAsync(&ea[b], sizeof(int32_t) * n, s));
      BOLA_TRY(make_kmajor_map(&mapA[b], aop[b], OZ_SLICES * n, true, 128));
      BOLA_TRY(make_kmajor_map(&mapA64[b], aop[b], OZ_SLICES * n, true, 64));
    }
    BOLA_TRY_CUDA(cudaMallocAsync(&bop, (size_t)OZ_SLICES * n * SNB * 2, s));
    BOLA_TRY_CUDA(cudaMallocAsync(&eb, sizeof(int32_t) * n, s));
    BOLA_TRY_CUDA(cudaMallocAsync(&sel, sizeof(double) * SNB * SNB, s));
    BOLA_TRY(make_kmajor_map(&mapB, bop, OZ_SLICES * n, true, 64));
    return 0;
  }
  const size_t esz = kind == 0 ? 2 : 4;
  const bool bf = kind == 0;
  // A operands in 128-row boxes (the update's rows) and 64-row boxes (as the
  // B side of a Cholesky update); B operands in 64-row boxes
  for (int b = 0; b < 2; ++b) {
    BOLA_TRY_CUDA(cudaMallocAsync(&aop[b], (size_t)n * SNB * esz, s));
    if (kind == 2) BOLA_TRY_CUDA(cudaMallocAsync(&aop_lo[b], (size_t)n * SNB * 4, s));
    BOLA_TRY(make_kmajor_map(&mapA[b], aop[b], n, bf));
    BOLA_TRY(make_kmajor_map(&mapAlo[b], kind == 2 ? aop_lo[b] : aop[b], n, bf));
    BOLA_TRY(make_kmajor_map(&mapA64[b], aop[b], n, bf, 64));
    BOLA_TRY(make_kmajor_map(&mapAlo64[b], kind == 2 ? aop_lo[b] : aop[b], n, bf, 64));
  }
  BOLA_TRY_CUDA(cudaMallocAsync(&bop, (size_t)n * SNB * esz, s));
  if (kind == 2) BOLA_TRY_CUDA(cudaMallocAsync(&bop_lo, (size_t)n * SNB * 4, s));
  BOLA_TRY(make_kmajor_map(&mapB, bop, n, bf, 64));
  BOLA_TRY(make_kmajor_map(&mapBlo, kind == 2 ? bop_lo : bop, n, bf, 64));
  return 0;
}

void MixedLU::release(cudaStream_t s) {
  for (void **p : {&aop[0], &aop[1], &bop, reinterpret_cast<void **>(&aop_lo[0]),
                   reinterpret_cast<void **>(&aop_lo[1]), reinterpret_cast<void **>(&bop_lo),
                   reinterpret_cast<void **>(&err), reinterpret_cast<void **>(&plan), reinterpret_cast<void **>(&track),
                   reinterpret_cast<void **>(&ea[0]),
                   reinterpret_cast<void **>(&ea[1]), reinterpret_cast<void **>(&eb),
                   reinterpret_cast<void **>(&sel)}) {
    if (*p) cudaFreeAsync(*p, s);
    *p = nullptr;
  }
  cap_n = 0;
}

void MixedLU::destroy() {
  release(nullptr);
  for (cudaEvent_t *e : {&ev_in, &ev_sw, &ev_wide, &ev_done}) {
    if (*e) cudaEventDestroy(*e);
    *e = nullptr;
  }
  for (cudaStream_t *st : {&sp, &su}) {
    if (*st) cudaStreamDestroy(*st);
    *st = nullptr;
  }
}

namespace {

// Width of the panel starting at j.
int panel_width(bool, int64_t n, int64_t j) { return (int)imin(SNB, n - j); }

}  // namespace

// Right-looking blocked LU of W (n x n), ipiv global 1-based, *info the first
// zero pivot (the factor is then unusable; the caller falls back).  Kinds 0-2:
// FP32 W and tc_update; kind 3: FP64 W and the exact-split oz_update.  Per
// step k: panel, swaps + U12 + B operand, the update of the next panel's
// columns (all on sp), then the update of the other columns on su, which
// overlaps panel k+1; the swaps of step k+1 wait for it.
template <typename T>
static int factor_lookahead(MixedLU &lu, cudaStream_t s, T *W, int64_t ldw, int32_t *ipiv, int32_t *info,
                            double give_up, int32_t *perm) {
  constexpr bool fp64 = std::is_same<T, double>::value;
  const int64_t n = lu.n;
  BOLA_TRY_CUDA(cudaEventRecord(lu.ev_in, s));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.sp, lu.ev_in, 0));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.su, lu.ev_in, 0));
  zero_i32<<<1, 1, 0, lu.sp>>>(info);
  track_init<<<1, 1, 0, lu.sp>>>(lu.track);
  if (perm != nullptr) iota32<<<(unsigned)cdiv(n, 256), 256, 0, lu.sp>>>(n, perm);
  BOLA_CHECK_LAUNCH();
  // su's first kernels read the flag too: they must see it initialised
  BOLA_TRY_CUDA(cudaEventRecord(lu.ev_in, lu.sp));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.su, lu.ev_in, 0));
  uint64_t *track = std::isinf(give_up) ? nullptr : lu.track;
  const int32_t *abort = track ? reinterpret_cast<const int32_t *>(track + 2) : nullptr;
  int jb = 0;
  bool wide_pending = false;
  for (int64_t j = 0, k = 0; j < n; j += jb, ++k) {
    jb = panel_width(fp64, n, j);
    const int64_t mp = n - j;
    const bool upd = j + jb < n;
    const int buf = (int)(k & 1);
    int32_t *plan_k = lu.plan + k * PLAN_STRIDE;  // this panel's moves, kept for apply_left_swaps
    if constexpr (fp64) {
      // pivot rows by tournament on FP32 copies, then the FP64 factorisation
      // of the selected block and of the rows below it
      double *Wp = W + j + j * ldw;
      int32_t *win = lu.plan + (int64_t)PLAN_STRIDE * cdiv(lu.cap_n, SNB);
      BOLA_TRY(launch_tpanel<double>(lu.sp, Wp, ldw, mp, jb, ipiv + j, (int32_t)j, info, nullptr, track, give_up,
                                     lu.err, win, lu.sel));
      {
        ProfScope prof(lu.sp, "panel_lu64", (double)jb * jb * jb * 2.0 / 3.0 + (double)(mp - jb) * jb * jb,
                       16.0 * (double)mp * jb);
        static bool attr = false;
        if (!attr) {
          BOLA_TRY_CUDA(cudaFuncSetAttribute(panel_lu64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PL_SMEM));
          attr = true;
        }
        const unsigned nA = mp > PL_SLOTS ? (unsigned)cdiv(mp - PL_SLOTS, PL_SLOTS) : 0u;
        StepLaunch L(dim3(nA + 1), dim3(PL_THREADS), PL_SMEM, lu.sp, true);
        BOLA_TRY_CUDA(cudaLaunchKernelEx(&L.cfg, panel_lu64, Wp, ldw, mp, jb, (int32_t)j, (const int32_t *)win,
                                         (const double *)lu.sel, plan_k, ipiv + j, info, track, give_up, lu.err,
                                         upd ? lu.aop[buf] : nullptr, lu.ea[buf], lu.cap_n));
      }
      BOLA_CHECK_LAUNCH();
    } else
      BOLA_TRY(launch_tpanel(lu.sp, W + j + j * ldw, ldw, mp, jb, ipiv + j, (int32_t)j, info, plan_k, track,
                             give_up, lu.err));
    // the row swaps reach every column: the previous wide update must be done
    if (wide_pending) BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.sp, lu.ev_wide, 0));
    wide_pending = false;
    if (n > jb) {  // (also the last panel: its moves reach the row permutation)
      ProfScope prof(lu.sp, fp64 ? "sswap_trsm64" : "sswap_trsm", (double)jb * jb * (double)(n - j - jb));
      // (the FP32 factors: one more CTA per 64 rows below the panel writes
      // the update's A operand)
      const int ncta = (int)imax(1, cdiv(n - j - jb, 8));
      const int nop = (!fp64 && upd) ? (int)cdiv(mp - jb, SNB) : 0;
      StepLaunch L(dim3((unsigned)(ncta + nop)), dim3(256), 0, lu.sp, true);
      BOLA_TRY_CUDA(cudaLaunchKernelEx(
          &L.cfg, sswap_trsm<T>, W, ldw, n, (int64_t)j, jb, (const int32_t *)plan_k, lu.kind,
          upd ? (void *)lu.bop : nullptr, fp64 ? (float *)nullptr : lu.bop_lo, fp64 ? lu.eb : (int32_t *)nullptr,
          lu.cap_n, abort, ncta, fp64 ? (void *)nullptr : lu.aop[buf], fp64 ? (float *)nullptr : lu.aop_lo[buf],
          perm));
      BOLA_CHECK_LAUNCH();
    }
    if (!upd) continue;
    const int64_t m2 = mp - jb, n2 = n - j - jb;
    const int64_t nb_next = imin((int64_t)panel_width(fp64, n, j + jb), n2);
    T *W22 = W + (j + jb) + (j + jb) * ldw;
    // (the next panel's columns follow the swap kernel on sp as its
    // programmatic dependent; the rest go to su)
    auto update = [&](cudaStream_t st, int64_t cols, int64_t boff) -> int {
      const bool pdl = st == lu.sp;
      if constexpr (fp64)
        return oz_update(st, m2, cols, lu.mapA[buf], lu.mapB, lu.cap_n, lu.cap_n, lu.ea[buf], lu.eb,
                         W22 + boff * ldw, ldw, lu.err, boff, abort, false, pdl);
      else
        return tc_update(st, lu.kind, m2, cols, lu.mapA[buf], lu.mapB, lu.mapAlo[buf], lu.mapBlo,
                         W22 + boff * ldw, ldw, lu.err, boff, abort, false, pdl);
    };
    BOLA_TRY(update(lu.sp, nb_next, 0));  // the next panel's columns
    if (n2 > nb_next) {
      BOLA_TRY_CUDA(cudaEventRecord(lu.ev_sw, lu.sp));
      BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.su, lu.ev_sw, 0));
      BOLA_TRY(update(lu.su, n2 - nb_next, nb_next));
      BOLA_TRY_CUDA(cudaEventRecord(lu.ev_wide, lu.su));
      wide_pending = true;
    }
  }
  // the interchanges on the columns left of each panel, all at once
  if (n > SNB) {
    ProfScope prof(lu.sp, "left_swaps");
    const size_t smem = ((sizeof(int32_t) * (size_t)(n - SNB) + 15) & ~(size_t)15) + sizeof(T) * (size_t)(n - SNB);
    static size_t attr = 0;
    if (smem > attr) {
      BOLA_TRY_CUDA(cudaFuncSetAttribute(apply_left_swaps<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr = smem;
    }
    apply_left_swaps<T><<<(unsigned)(cdiv(n, SNB) - 1), 512, smem, lu.sp>>>(W, ldw, n, lu.plan, abort);
    BOLA_CHECK_LAUNCH();
  }
  if (wide_pending) BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.sp, lu.ev_wide, 0));
  BOLA_TRY_CUDA(cudaEventRecord(lu.ev_done, lu.sp));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(s, lu.ev_done, 0));
  return 0;
}

int MixedLU::factor(cudaStream_t s, float *W, int64_t ldw, int32_t *ipiv, int32_t *info, double give_up,
                    int32_t *perm) {
  return factor_lookahead<float>(*this, s, W, ldw, ipiv, info, give_up, perm);
}

int MixedLU::factor64(cudaStream_t s, double *W, int64_t ldw, int32_t *ipiv, int32_t *info, double give_up,
                      int32_t *perm) {
  return factor_lookahead<double>(*this, s, W, ldw, ipiv, info, give_up, perm);
}

}  // namespace bola

// The low-precision LU alone, for tests and profiling: W (n x n FP32,
// column-major, ld ldw) is replaced by its factors (unit-lower L below the
// diagonal, U on and above), ipiv (device, 1-based, LAPACK order) and *info
// (device: the first exact-zero pivot, 1-based, or 0).  Synchronous.
extern "C" int bola_sgetrf_mixed(int kind, int64_t n, float *w, int64_t ldw, int32_t *ipiv, int32_t *info,
                                 bola_stream_t stream) {
  using namespace bola;
  if (kind < 0 || kind > 2) return -1;
  if (n < 0 || n > 8192) return -2;
  if (ldw < imax(1, n)) return -4;
  if (n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  MixedLU lu;
  int st = lu.reserve(n, kind, s);
  if (st == 0) st = lu.factor(s, w, ldw, ipiv, info);
  int32_t err = 0;
  if (st == 0 && lu.err) st = cudaMemcpyAsync(&err, lu.err, sizeof err, cudaMemcpyDeviceToHost, s) == cudaSuccess ? 0 : BOLA_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess && st == 0) st = fail(BOLA_ERR_CUDA, "bola_sgetrf_mixed: %s", cudaGetErrorString(cudaGetLastError()));
  lu.destroy();
  if (st == 0 && err != 0) st = fail(BOLA_ERR_CUDA, "mixed LU: a bounded wait expired (code %d)", err);
  return st;
}
