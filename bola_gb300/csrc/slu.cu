// slu.cu — the low-precision LU of the mixed-precision solver (no BOLA
// counterpart; it preconditions the FP64 refinement in ir.cu).
//
// A (FP64) is scaled per 64-column block by a power of two (exact) and
// rounded to the working matrix W: FP32 (factor kinds 0-2) or FP64 (kind 3).
// Blocked right-looking LU, NB = 64 = the K of the tensor-core update:
//   tpanel_kernel   FP32 W: the (n-j) x 64 panel on a cluster of <= 16 CTAs,
//                   rows in shared memory, pivots chosen by tournament over
//                   groups of 8 columns (one cluster exchange per group);
//   spanel_kernel   FP64 W: the same panel with column-by-column partial
//                   pivoting (each CTA pushes its candidate row into every
//                   CTA's shared memory with st.async, per column).
//   Both write L21 as the update's K-major A operand (bf16, tf32 hi/lo, or
//   the exact bf16 slices of the FP64-accurate factor).
//   sswap_trsm      the 64 interchanges on every other column, U12 = L11^-1 A12
//                   and the K-major B operand.
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
constexpr int SPT = 256;  // threads per panel CTA
constexpr int SMAXC = 16;

template <typename T>
struct alignas(16) SSlot {
  uint32_t k0, k1, k2, pad;  // pivot key (see PKey)
  T v[SNB];                  // the candidate row
};

// Bulk copy of `bytes` (a multiple of 16) from this CTA's shared memory into
// another CTA's (cluster addresses dst and bar), completing on the
// receiver's mbarrier; the issuing thread commits it as a bulk group.
__device__ __forceinline__ void bulk_push(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "r"(sm100::smem_u32(src)), "r"(bytes), "r"(bar)
      : "memory");
}

// Pivot key, compared lexicographically: the bits of |v| (high word, low
// word; the low word is 0 for FP32) and ~row, so the largest magnitude wins
// and ties go to the lowest row; a NaN never wins.
struct PKey {
  uint32_t a, b, c;
};
__device__ __forceinline__ bool pk_less(const PKey &x, const PKey &y) {
  return x.a != y.a ? x.a < y.a : (x.b != y.b ? x.b < y.b : x.c < y.c);
}
__device__ __forceinline__ PKey pk_make(double v, int g) {
  // |v| and the NaN test on the bits: an FP64 comparison would take an FP64 pipe slot
  uint64_t u = (uint64_t)__double_as_longlong(v) & 0x7fffffffffffffffull;
  u = u > 0x7ff0000000000000ull ? 0ull : u;
  return PKey{(uint32_t)(u >> 32), (uint32_t)u, 0xFFFFFFFFu - (uint32_t)g};
}
__device__ __forceinline__ PKey pk_warp_max(const PKey &k) {
  const uint32_t a = __reduce_max_sync(0xffffffffu, k.a);
  const uint32_t b = __reduce_max_sync(0xffffffffu, k.a == a ? k.b : 0u);
  const uint32_t c = __reduce_max_sync(0xffffffffu, (k.a == a && k.b == b) ? k.c : 0u);
  return PKey{a, b, c};
}

// ---- panel arithmetic ---------------------------------------------------------
// The column-by-column panel kernel works on elements of type S in shared
// memory, loaded from and stored to W of type G, through these operations
// (the FP64-accurate factor's panel).
struct PanelF64 {
  using S = double;
  using G = double;
  static constexpr bool kFP64 = true;
  __device__ static S zero() { return 0.0; }
  __device__ static S load(G x) { return x; }
  __device__ static G store(S x) { return x; }
  __device__ static S mul(S a, S b) { return a * b; }
  __device__ static S fnms(S z, S x, S y) { return fma(-x, y, z); }
  __device__ static bool is_zero(S p) { return !nonzero64(p); }
  __device__ static S recip(S p) { return nonzero64(p) ? 1.0 / p : 0.0; }
  __device__ static PKey key(S v, int g) { return pk_make(v, g); }
  __device__ static double to_double(S v) { return v; }
  __device__ static uint64_t abs_bits(S v) { return (uint64_t)__double_as_longlong(v) & 0x7fffffffffffffffull; }
  __device__ static bool is_nan_bits(uint64_t b) { return b > 0x7ff0000000000000ull; }
  __device__ static uint64_t bits_to_double_bits(uint64_t b) { return b; }
};


// Row pitch of a panel held in shared memory: at least R + 1 and a multiple
// of the 16-byte vector (4 floats or 2 doubles), so that a lane can move V
// consecutive rows of a column in one access.
template <typename T>
__host__ __device__ constexpr int panel_pitch(int64_t R) {
  return (int)(((R + (int64_t)(16 / sizeof(T))) / (int64_t)(16 / sizeof(T))) * (int64_t)(16 / sizeof(T)));
}
__device__ __forceinline__ void vload(double (&v)[2], const double *p) {
  const double2 t = *reinterpret_cast<const double2 *>(p);
  v[0] = t.x; v[1] = t.y;
}
__device__ __forceinline__ void vstore(double *p, const double (&v)[2]) {
  *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
}

// Panel LU of W[0:mp, 0:jb] (W points at the panel's top-left).  ipiv gets
// global 1-based rows (col0 + local + 1).  CTA cr of the cluster owns panel
// rows [cr*R, cr*R + R), kept in shared memory column-major with an odd
// pitch (R + 1) so that both a thread walking its row and a warp walking a
// column are conflict-free.
//
// Per column j: pivot search in column j, one CTA barrier, every warp pushes
// the CTA's candidate row (and row j if the CTA owns it) into its share of
// the CTAs with asynchronous remote stores that count their bytes on the
// receiver's mbarrier (st.async), one CTA barrier; then, while the other
// CTAs' pushes arrive, the rank-1 update of pivot j-1 on columns j+1..
// (deferred from the previous column); a wait on this CTA's own mbarrier for
// every CTA's push (no cluster-wide barrier: a CTA pushes column j+1 only
// after it has read column j's slots, which is what makes the double-buffered
// slots safe); every CTA picks the same winner from its own slots and brings
// the pushed rows up to date (they left before pivot j-1's deferred update
// reached their columns > j: the same fmaf the owner does); swap; one CTA
// barrier; the update of column j+1 only (the next pivot column).
// Multipliers of column j are scaled when column j+1 is searched.  Waits are
// bounded: a push that never lands sets *err and ends the panel.

template <typename P>
__global__ void __launch_bounds__(SPT)
spanel_kernel(typename P::G *W, int64_t ldw, int64_t mp, int jb, int32_t *ipiv, int32_t col0, int32_t *info, int kind,
              void *aop, float *aop_lo, int32_t *aexp, int64_t cap, int64_t R, int32_t *plan, uint64_t *track,
              double give_up, int32_t *err) {
  cg::cluster_group cluster = cg::this_cluster();
  // An abandoned factorisation: the flag was set by an earlier panel on this
  // stream, so every CTA of the cluster reads the same value.  Identity
  // pivots keep ipiv valid for the kernels after the factorisation that
  // compose it (the factor itself is discarded).
  if (track != nullptr && *(volatile const int32_t *)(track + 2) != 0) {
    if (cluster.block_rank() == 0)
      for (int t = threadIdx.x; t < jb; t += blockDim.x) ipiv[t] = col0 + t + 1;
    return;
  }
  const int C = (int)cluster.num_blocks();
  const int cr = (int)cluster.block_rank();
  using T = typename P::S;
  __shared__ SSlot<T> slots[2][SMAXC];
  __shared__ T rowj[2][SNB];
  __shared__ T piv[2][SNB];   // pivot rows, up to date (piv[par] = column j's)
  __shared__ T oldj[SNB];     // the old row j, up to date (goes to the pivot's place)
  __shared__ PKey wkey[SPT / 32];
  __shared__ T sinv;          // 1 / pivot of the current column
  __shared__ uint64_t xbar[2];  // completes when every CTA's push for a column has landed here
  __shared__ int sfail;
  extern __shared__ __align__(16) unsigned char sp_raw[];
  T *sp = reinterpret_cast<T *>(sp_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int RP = panel_pitch<T>(R);
  const int r0 = (int)(cr * R);
  const int r1 = (int)imin(mp, r0 + R);
  const int nr = r1 > r0 ? r1 - r0 : 0;
  // element (row il, column c) of this CTA's rows, in shared memory
  auto PE = [&](int c, int il) -> T & { return sp[c * RP + il]; };
  const int ns = nr;

  // a thread's rows, 16 columns at a time, all of those loads in flight together
  for (int il0 = tid; il0 < ns; il0 += 2 * SPT) {
    const int il1 = il0 + SPT;
    for (int c0 = 0; c0 < jb; c0 += 16) {
      typename P::G t0[16], t1[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        t0[c] = c0 + c < jb ? W[(r0 + il0) + (int64_t)(c0 + c) * ldw] : typename P::G(0);
        t1[c] = (il1 < ns && c0 + c < jb) ? W[(r0 + il1) + (int64_t)(c0 + c) * ldw] : typename P::G(0);
      }
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        if (c0 + c >= jb) break;
        sp[(c0 + c) * RP + il0] = P::load(t0[c]);
        if (il1 < ns) sp[(c0 + c) * RP + il1] = P::load(t1[c]);
      }
    }
  }
  if (tid == 0) {
    sm100::mbar_init(&xbar[0], 1);
    sm100::mbar_init(&xbar[1], 1);
    sm100::fence_mbar_init();
    sfail = 0;
  }
  __syncthreads();
  cluster.sync();  // every CTA runs, its mbarriers initialised, before the first push
  // bytes that land in this CTA per column: a slot from every CTA, row j from its owner
  constexpr uint32_t SLOT_BYTES = 16 + SNB * sizeof(T), ROW_BYTES = SNB * sizeof(T);
  const uint32_t xbytes = (uint32_t)C * SLOT_BYTES + ROW_BYTES;
  bool failed = false;

  T inv = P::zero();  // 1 / pivot of the previous column
  // |u_jj| of this panel's pivots as ordered integer bits (NaN ignored, as
  // fmax/fmin ignore it): thread 0 of CTA 0 only, on the integer pipe
  uint64_t umax = 0, umin = ~0ull;
  for (int j = 0; j < jb; ++j) {
    const int par = j & 1;
    const T *pprev = piv[par ^ 1];
    // this column's phase of xbar[par] (its previous phase, column j-2, was
    // waited for by every thread): expect the pushes
    if (tid == 0) sm100::mbar_arrive_expect_tx(&xbar[par], xbytes);
    // -- the multipliers of column j-1, then this CTA's pivot candidate in
    // column j: key = (|v| bits, ~row), max wins, ties -> lowest row
    PKey best = PKey{0u, 0u, 0u};
    for (int il = tid; il < nr; il += SPT) {
      const int g = r0 + il;
      if (j > 0 && g >= j) PE(j - 1, il) = P::mul(PE(j - 1, il), inv);
      if (g < j) continue;
      const PKey k = P::key(PE(j, il), g);
      if (pk_less(best, k)) best = k;
    }
    best = pk_warp_max(best);
    if (lane == 0) wkey[warp] = best;
    __syncthreads();
    // -- every warp pushes the candidate (and row j if owned) to its share of the CTAs
    {
      PKey ck = wkey[0];
#pragma unroll
      for (int w = 1; w < SPT / 32; ++w)
        if (pk_less(ck, wkey[w])) ck = wkey[w];
      const int gl = ck.c ? (int)(0xFFFFFFFFu - ck.c) - r0 : -1;  // local row of the candidate
      const bool own_j = j >= r0 && j < r1;
      const int jl = j - r0;
      T c0 = P::zero(), c1 = P::zero(), j0v = P::zero(), j1v = P::zero();
      if (gl >= 0) {
        c0 = lane < jb ? PE(lane, gl) : P::zero();
        c1 = lane + 32 < jb ? PE(lane + 32, gl) : P::zero();
      }
      if (own_j) {
        j0v = lane < jb ? PE(lane, jl) : P::zero();
        j1v = lane + 32 < jb ? PE(lane + 32, jl) : P::zero();
      }
      for (int d = warp; d < C; d += SPT / 32) {
        const uint32_t rbar = sm100::cluster_addr(&xbar[par], d);
        const uint32_t rs = sm100::cluster_addr(&slots[par][cr], d);
        if (lane == 0) sm100::st_async4(rs, ck.a, ck.b, ck.c, 0u, rbar);
        sm100::st_async(rs + 16 + lane * (uint32_t)sizeof(T), c0, rbar);
        sm100::st_async(rs + 16 + (lane + 32) * (uint32_t)sizeof(T), c1, rbar);
        if (own_j) {
          const uint32_t rj = sm100::cluster_addr(&rowj[par][0], d);
          sm100::st_async(rj + lane * (uint32_t)sizeof(T), j0v, rbar);
          sm100::st_async(rj + (lane + 32) * (uint32_t)sizeof(T), j1v, rbar);
        }
      }
    }
    __syncthreads();  // the rows are read before the deferred update changes them
    // -- the deferred rank-1 update of pivot j-1 on columns j+1..jb-1, rows >= j:
    // lanes walk rows, warps take every 8th column; the pivot-row values sit
    // in registers, so a thread's 8 loads are all in flight together
    if (j > 0 && j + 1 < jb) {
      T pr[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int c = j + 1 + warp + 8 * q;
        pr[q] = c < jb ? pprev[c] : P::zero();
      }
      // 16-byte shared-memory accesses: a lane takes V consecutive rows
      constexpr int V = 16 / (int)sizeof(T);
      const int ib = j > r0 ? j - r0 : 0;
      for (int il0 = (ib & ~(V - 1)) + lane * V; il0 < nr; il0 += 32 * V) {
        T l[V];
        vload(l, &sp[(j - 1) * RP + il0]);
        bool on[V];
#pragma unroll
        for (int e = 0; e < V; ++e) on[e] = il0 + e >= ib && il0 + e < nr;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int c = j + 1 + warp + 8 * q;
          if (c >= jb) continue;
          T v[V];
          vload(v, &sp[c * RP + il0]);
#pragma unroll
          for (int e = 0; e < V; ++e)
            if (on[e]) v[e] = P::fnms(v[e], l[e], pr[q]);
          vstore(&sp[c * RP + il0], v);
        }
      }
    }
    // every CTA's push for this column has landed (bounded: a missing push
    // sets the error flag and ends the panel, never a hang)
    {
      const bool ok = sm100::bounded_wait(&xbar[par], (uint32_t)(j >> 1) & 1u);
      if (!ok) sfail = 1;
      __syncthreads();
      if (sfail) {
        if (tid == 0) atomicExch(err, 5);
        failed = true;
        break;
      }
    }
    // -- the winner, identical in every CTA: lane s reads slot s, warp max
    PKey wk;
    int ws = 0;
    {
      const PKey k = lane < C ? PKey{slots[par][lane].k0, slots[par][lane].k1, slots[par][lane].k2} : PKey{0u, 0u, 0u};
      wk = pk_warp_max(k);
      const unsigned m = __ballot_sync(0xffffffffu, lane < C && k.a == wk.a && k.b == wk.b && k.c == wk.c);
      ws = m ? __ffs(m) - 1 : 0;
    }
    const int jp = wk.c ? (int)(0xFFFFFFFFu - wk.c) : j;
    const T *raw = wk.c ? slots[par][ws].v : rowj[par];
    T *pcur = piv[par];
    // the pushed rows, brought up to date: columns > j still lack pivot j-1
    if (tid < jb) {
      T pv_ = raw[tid], ov = rowj[par][tid];
      if (j > 0 && tid > j) {
        pv_ = P::fnms(pv_, raw[j - 1], pprev[tid]);
        ov = P::fnms(ov, rowj[par][j - 1], pprev[tid]);
      }
      pcur[tid] = pv_;
      oldj[tid] = ov;
      if (tid == j) sinv = P::recip(pv_);  // once per CTA, not once per thread
    }
    __syncthreads();
    const T pv = pcur[j];
    if (cr == 0 && tid == 0) {
      ipiv[j] = col0 + jp + 1;
      const uint64_t ab = P::abs_bits(pv);
      if (!P::is_nan_bits(ab)) {
        umax = ab > umax ? ab : umax;
        umin = ab < umin ? ab : umin;
      }
    }
    inv = sinv;
    if (P::is_zero(pv)) {
      if (cr == 0 && tid == 0) atomicCAS(info, 0, col0 + j + 1);
    }
    if (jp != j && tid < jb) {
      if (j >= r0 && j < r1) PE(tid, j - r0) = pcur[tid];
      if (jp >= r0 && jp < r1) PE(tid, jp - r0) = oldj[tid];
    }
    __syncthreads();
    // -- the next pivot column now (the rest of this update is deferred);
    // same row-to-thread map as the search, so no barrier before it
    if (j + 1 < jb) {
      const T pj1 = pcur[j + 1];
      for (int il = tid; il < nr; il += SPT) {
        if (r0 + il <= j) continue;
        T &x = PE(j + 1, il);
        x = P::fnms(x, P::mul(PE(j, il), inv), pj1);
      }
    }
  }
  if (!failed) {  // (after a failed exchange the error flag fails the whole call)
  // the last column's multipliers
  for (int il = tid; il < nr; il += SPT)
    if (r0 + il >= jb) PE(jb - 1, il) = P::mul(PE(jb - 1, il), inv);
  __syncthreads();
  if (track != nullptr && cr == 0 && tid == 0) {
    // the running extent of |u_ii| and the give-up test (the spread only grows
    // as pivots are added, so giving up early decides as the whole factor would)
    if (umin != ~0ull) {
      const uint64_t mx = P::bits_to_double_bits(umax), mn = P::bits_to_double_bits(umin);
      if (mx > track[0]) track[0] = mx;
      if (mn < track[1]) track[1] = mn;
    }
    const double gmx = __longlong_as_double((long long)track[0]), gmn = __longlong_as_double((long long)track[1]);
    const double spread = gmn > 0.0 ? gmx / gmn : INFINITY;
    if (give_up_now(spread, give_up, col0 + jb, col0 + mp)) *(volatile int32_t *)(track + 2) = 1;
  }

  // -- write back the panel and the update's A operand (rows below the panel)
  for (int il = tid; il < ns; il += SPT) {
    typename P::G *wr = W + (r0 + il);
#pragma unroll 8
    for (int c = 0; c < jb; ++c) wr[(int64_t)c * ldw] = P::store(sp[c * RP + il]);
  }
  if (plan != nullptr && cr == 0 && warp == 0) {
    // the panel's interchanges as "row rows[t] takes the old row src[t]",
    // composed once here for the swap kernel that follows
    __syncwarp();
    SwapPlan p;
    p.ix0 = 0;
    p.i1 = col0 + 1;
    p.i2 = col0 + jb;
    p.i_inc = 1;
    p.incx = 1;
    const int cnt = compose_swaps_warp<4, int32_t>(p, ipiv, plan + 1, plan + 1 + 2 * SNB);
    if (lane == 0) plan[0] = cnt;
  }
  if (aop != nullptr) {
    for (int il = tid; il < nr; il += SPT) {
      const int g = r0 + il;
      if (g < jb) continue;
      if constexpr (!P::kFP64) {
        float v[SNB];
#pragma unroll
        for (int c = 0; c < SNB; ++c) v[c] = c < jb ? PE(c, il) : 0.f;
        write_operand_row(kind, aop, aop_lo, g - jb, v);
      } else {
        // exact bf16 slices of the row (FP64 factor): exponent, then 8 K values at a time
        uint64_t mb = 0;
        for (int c = 0; c < jb; ++c) {
          const uint64_t mc = oz_mag(P::to_double(PE(c, il)));
          mb = mc > mb ? mc : mb;
        }
        const int e = oz_exponent(mb);
        aexp[g - jb] = e;
        __nv_bfloat16 *out = static_cast<__nv_bfloat16 *>(aop);
        for (int c0 = 0; c0 < SNB; c0 += 8) {
          __align__(16) __nv_bfloat16 q[OZ_SLICES][8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            __nv_bfloat16 t8[OZ_SLICES];
            oz_slices(c0 + u < jb ? P::to_double(PE(c0 + u, il)) : 0.0, e, t8);
#pragma unroll
            for (int t = 0; t < OZ_SLICES; ++t) q[t][u] = t8[t];
          }
#pragma unroll
          for (int t = 0; t < OZ_SLICES; ++t)
            *reinterpret_cast<uint4 *>(out + ((int64_t)t * cap + (g - jb)) * SNB + c0) =
                *reinterpret_cast<const uint4 *>(q[t]);
        }
      }
    }
  }
  }
  cluster.sync();  // no CTA leaves while another may still push into it
}

// ---- tournament panel (the FP32 factors) ----------------------------------------
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

// Partial pivoting over gw <= TG columns of the candidates a warp holds
// (candidate l + 32 r sits in row r of lane l).  The pivot key is |v| with
// its 8 lowest bits replaced by 255 - candidate, so that one warp reduction
// finds the pivot (the lowest mantissa bits do not matter for the pivot's
// quality; ties go to the lowest candidate; a NaN never wins).  The column
// loop is not unrolled (code size: the panel's phases would otherwise keep
// missing the instruction cache); instead the current column always sits in
// register slot 0 and the remaining ones shift down after each step.  Writes
// the selected candidates in order to sel[] (shared memory, lane 0) and
// returns their count.  RECORD: each candidate's multipliers go to
// Lsm[candidate * TG + step] (shared), the selected rows' ones to Lrec[t][s]
// (s < t), and the pivot rows' eliminated values in group column t + k to
// Urec[(t + k) * uk + t].
template <int RPL, bool RECORD>
__device__ __forceinline__ int warp_gepp(float (&v)[RPL][TG], bool (&live)[RPL], int gw, int *sel, float *Lsm,
                                         float (*Lrec)[TG], float *Urec, int uk) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int cnt = 0;
#pragma unroll 1
  for (int t = 0; t < gw; ++t) {
    uint32_t key = 0u;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const float x = fabsf(v[r][0]);
      const uint32_t a = x == x ? __float_as_uint(x) : 0u;
      const uint32_t k = (a & ~0xFFu) | (uint32_t)(255 - (lane + 32 * r));
      key = (live[r] && k > key) ? k : key;
    }
    const uint32_t mk = __reduce_max_sync(FULL, key);
    if (mk == 0u) break;  // no live candidate left (a live one has a key >= 128)
    const int slot = 255 - (int)(mk & 0xFFu);
    const int wl = slot & 31, wr = slot >> 5;
    float pv[TG];
#pragma unroll
    for (int k = 0; k < TG; ++k) {
      float x = v[0][k];
#pragma unroll
      for (int r = 1; r < RPL; ++r)
        if (wr == r) x = v[r][k];
      pv[k] = __shfl_sync(FULL, x, wl);
    }
    if (lane == 0) sel[t] = slot;
    if (lane == wl) {
#pragma unroll
      for (int r = 0; r < RPL; ++r)
        if (r == wr) live[r] = false;
    }
    if (RECORD) {
      if (lane < t) Lrec[t][lane] = Lsm[slot * TG + lane];
      if (lane < TG && lane < gw - t) {
        float x = pv[0];
#pragma unroll
        for (int k = 1; k < TG; ++k)
          if (lane == k) x = pv[k];
        Urec[(t + lane) * uk + t] = x;
      }
    }
    const float inv = pv[0] != 0.f ? __frcp_rn(pv[0]) : 0.f;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const float l = v[r][0] * inv;
      if (RECORD && live[r]) Lsm[(lane + 32 * r) * TG + t] = l;
#pragma unroll
      for (int k = 1; k < TG; ++k) v[r][k - 1] = live[r] ? fmaf(-l, pv[k], v[r][k]) : v[r][k];
      v[r][TG - 1] = 0.f;
    }
    ++cnt;
  }
  __syncwarp();
  return cnt;
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

__global__ void __launch_bounds__(TPT, 1)
tpanel_kernel(float *W, int64_t ldw, int64_t mp, int jb, int32_t *ipiv, int32_t col0, int32_t *info, int kind,
              void *aop, float *aop_lo, int64_t R, int32_t *plan, uint64_t *track, double give_up, int32_t *err) {
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
  __shared__ int32_t cand1[TPT / 32][TG];  // each warp's nominees (local rows, -1: none)
  __shared__ int32_t cand2[TG];            // the CTA's nominees
  __shared__ int32_t win[SNB];             // panel row of the pivot of each column
  __shared__ int32_t wslot[TG];            // the group's pivots as slot indices
  __shared__ float Lg[TG][TG];             // the group pivots' multipliers within the group
  __shared__ __align__(16) float UgT[2][SNB][TG];  // U rows of a group's pivots, transposed (two groups)
  __shared__ float invp[TG];
  __shared__ int32_t posin[SNB], at_[SNB], ipg[SNB];  // interchange bookkeeping (CTA 0)
  __shared__ int sfail;
  __shared__ TSlot stage[TG];              // this CTA's nominees, as they are pushed
  __shared__ int32_t selw[TPT / 32][TG];   // pivot search outputs (candidate order)
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
        t[r][c] = (il < nr && c0 + c < jb) ? W[(r0 + il) + (int64_t)(c0 + c) * ldw] : 0.f;
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
    // -- 1. each warp's nominees from its own rows (the group's columns are current)
    {
      float v[TRPL][TG];
      bool live[TRPL];
#pragma unroll
      for (int r = 0; r < TRPL; ++r) {
        const int il = warp * 32 + lane + TPT * r;
        live[r] = il < nr && rstate[il] < 0;
#pragma unroll
        for (int k = 0; k < TG; ++k) v[r][k] = live[r] ? sp[(c0 + k) * RP + il] : 0.f;
      }
      const int cnt = warp_gepp<TRPL, false>(v, live, gw, selw[warp], nullptr, nullptr, nullptr, 0);
      if (lane < TG) {
        const int sl = selw[warp][lane];
        cand1[warp][lane] = lane < cnt ? warp * 32 + (sl & 31) + TPT * (sl >> 5) : -1;
      }
    }
    __syncthreads();
    // -- 2. the CTA's nominees from the warps' (warp 0)
    if (warp == 0) {
      constexpr int NC1 = (TPT / 32) * TG;  // 64 candidates: 2 per lane
      float v[NC1 / 32][TG];
      bool live[NC1 / 32];
      int cil[NC1 / 32];
#pragma unroll
      for (int r = 0; r < NC1 / 32; ++r) {
        const int ci = lane + 32 * r;
        cil[r] = cand1[ci / TG][ci % TG];
        live[r] = cil[r] >= 0;
#pragma unroll
        for (int k = 0; k < TG; ++k) v[r][k] = live[r] ? sp[(c0 + k) * RP + cil[r]] : 0.f;
      }
      const int cnt = warp_gepp<NC1 / 32, false>(v, live, gw, selw[0], nullptr, nullptr, nullptr, 0);
      if (lane < TG) {
        const int ci = selw[0][lane];
        cand2[lane] = lane < cnt ? cand1[ci / TG][ci % TG] : -1;
      }
      // the previous group's bulk pushes have read the staging slots
      if (lane < C) sm100::bulk_wait_read0();
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
    if (g > 0) {
      const float(*U)[TG] = UgT[ub ^ 1];
#pragma unroll
      for (int r = 0; r < TRPL; ++r) {
        const int il = tid + TPT * r;
        if (il >= nr || rstate[il] >= 0) continue;
        float l[TG];
#pragma unroll
        for (int s2 = 0; s2 < TG; ++s2) l[s2] = sp[(pb + s2) * RP + il];
        for (int k = c0 + TG; k < SNB; ++k) {
          const float4 u0 = *reinterpret_cast<const float4 *>(&U[k][0]);
          const float4 u1 = *reinterpret_cast<const float4 *>(&U[k][4]);
          sp[k * RP + il] = rank8(sp[k * RP + il], l, u0, u1);
        }
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
    // -- 5. the group's pivots from all nominees, the same in every CTA (warp
    // 0), while the other warps bring every pushed row's columns right of the
    // group up to date with the previous group's update (the pushed
    // multipliers of that group are its first 8 values), in place
    if (warp == 0) {
      constexpr int NC3 = SMAXC * TG / 32;  // up to 128 candidates: 4 per lane
      float v[NC3][TG];
      bool live[NC3];
#pragma unroll
      for (int r = 0; r < NC3; ++r) {
        const int ci = lane + 32 * r;
        live[r] = ci < C * gw && sl[ci].row != 0xFFFFFFFFu;
#pragma unroll
        for (int k = 0; k < TG; ++k) v[r][k] = live[r] ? sl[ci].v[c0 - pb + k] : 0.f;
      }
      const int cnt = warp_gepp<NC3, true>(v, live, gw, selw[0], Lsm, Lg, &UgT[ub][c0][0], TG);
      // the panel always has at least gw rows that are not pivots yet, so
      // cnt == gw; a shortfall would mean a corrupted exchange
      if (cnt < gw && lane == 0) atomicExch(err, 6);
      if (lane < gw) {
        const int s2 = selw[0][lane];
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
    } else if (g > 0) {
      TSlot *slw = slots + (size_t)par * C * TG;
      const float(*U)[TG] = UgT[ub ^ 1];
      const int nk = SNB - c0 - gw;
      for (int e = tid - 32; e < C * gw * nk; e += TPT - 32) {
        const int ci = e / nk, k = c0 + gw + e % nk;
        float l[TG];
#pragma unroll
        for (int s2 = 0; s2 < TG; ++s2) l[s2] = slw[ci].v[s2];
        slw[ci].v[k - pb] = rank8(slw[ci].v[k - pb], l, *reinterpret_cast<const float4 *>(&U[k][0]),
                                  *reinterpret_cast<const float4 *>(&U[k][4]));
      }
    }
    __syncthreads();
    if (win[c0 + gw - 1] < 0) {  // (err is set) leave the group loop uniformly
      failed = true;
      break;
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
        if (pv == 0.f) atomicCAS(info, 0, col0 + c0 + t + 1);
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
#pragma unroll
    for (int r = 0; r < TRPL; ++r) {
      const int il = tid + TPT * r;
      if (il >= nr) continue;
      if (rstate[il] >= 0) continue;  // a pivot row (of this group: written above)
      float l[TG];
#pragma unroll
      for (int s2 = 0; s2 < TG; ++s2) {
        l[s2] = 0.f;
        if (s2 >= gw) continue;
        float a = sp[(c0 + s2) * RP + il];
#pragma unroll
        for (int q = 0; q < s2; ++q) a = fmaf(-l[q], UgT[ub][c0 + s2][q], a);
        l[s2] = a * invp[s2];
        sp[(c0 + s2) * RP + il] = l[s2];
      }
      const int k1 = (int)imin(SNB, c0 + 2 * TG);
      for (int k = c0 + TG; k < k1; ++k) {
        const float4 u0 = *reinterpret_cast<const float4 *>(&UgT[ub][k][0]);
        const float4 u1 = *reinterpret_cast<const float4 *>(&UgT[ub][k][4]);
        sp[k * RP + il] = rank8(sp[k * RP + il], l, u0, u1);
      }
    }
    __syncthreads();
  }
  if (!failed) {
    // -- the interchanges (CTA 0): LAPACK's sequence of row swaps that puts
    // the pivot of column j in row j, from the pivot list.  Rows below the
    // panel's first jb never move until they become a pivot; rows among the
    // first jb are tracked: at_[q] = the row now in position q < jb,
    // posin[x] = the position of original row x < jb.
    if (cr == 0 && tid == 0) {
      for (int x = 0; x < jb; ++x) posin[x] = at_[x] = x;
      for (int j = 0; j < jb; ++j) {
        const int x = win[j];
        const int q = x < jb ? posin[x] : x;
        ipg[j] = col0 + q + 1;
        const int r = at_[j];
        if (r != x) {
          if (q < jb) at_[q] = r;
          posin[r] = q;
        }
        at_[j] = x;
        if (x < jb) posin[x] = j;
      }
      for (int j = 0; j < jb; ++j) ipiv[j] = ipg[j];
    }
    __syncthreads();
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
    // final position of each of this CTA's rows
    auto dest = [&](int il) -> int {
      const int st = rstate[il];
      if (st >= 0) return st;
      if (cr == 0 && il < jb) return posin[il];
      return r0 + il;
    };
    // -- write back the panel, each row to its final position
#pragma unroll
    for (int r = 0; r < TRPL; ++r) {
      const int il = tid + TPT * r;
      if (il >= nr) continue;
      float *wr = W + dest(il);
#pragma unroll 8
      for (int c = 0; c < jb; ++c) wr[(int64_t)c * ldw] = sp[c * RP + il];
    }
    if (plan != nullptr && cr == 0 && warp == 0) {
      // the interchanges as "row rows[t] takes the old row src[t]" for the swap kernel
      SwapPlan p;
      p.ix0 = 0;
      p.i1 = col0 + 1;
      p.i2 = col0 + jb;
      p.i_inc = 1;
      p.incx = 1;
      const int cnt = compose_swaps_warp<4, int32_t>(p, ipg, plan + 1, plan + 1 + 2 * SNB);
      if (lane == 0) plan[0] = cnt;
    }
    if (aop != nullptr) {  // rows below the panel's top: the update's K-major A operand
      for (int il = tid; il < nr; il += TPT) {
        const int dst = dest(il);
        if (dst < jb) continue;
        float v[SNB];
#pragma unroll
        for (int c = 0; c < SNB; ++c) v[c] = c < jb ? sp[c * RP + il] : 0.f;
        write_operand_row(kind, aop, aop_lo, dst - jb, v);
      }
    }
  }
  if (tid < C) sm100::bulk_wait_read0();  // this CTA's last pushes have read its staging slots
  cluster.sync();  // no CTA leaves while another may still push into it
}

int launch_tpanel(cudaStream_t s, float *W, int64_t ldw, int64_t mp, int jb, int32_t *ipiv, int32_t col0,
                  int32_t *info, int kind, void *aop, float *aop_lo, int32_t *plan, uint64_t *track, double give_up,
                  int32_t *err) {
  const int C = (int)imin(SMAXC, imax(1, cdiv(mp, TPT)));
  const int64_t R = cdiv(mp, C);
  // CTA 0 must hold the panel's first jb rows (the interchange bookkeeping)
  if (R > (int64_t)TPT * TRPL || R < jb)
    return fail(BOLA_ERR_UNSUPPORTED, "mixed LU: panel of %lld x %d not supported", (long long)mp, jb);
  const size_t smem = tpanel_smem(R, C);
  static bool attr = false;
  if (!attr) {
    BOLA_TRY_CUDA(cudaFuncSetAttribute(tpanel_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    BOLA_TRY_CUDA(cudaFuncSetAttribute(tpanel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)tpanel_smem(TPT * TRPL, SMAXC)));
    attr = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C, 1, 1);
  cfg.blockDim = dim3(TPT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  ProfScope prof(s, "tpanel", (double)mp * jb * jb, 8.0 * (double)mp * jb);
  BOLA_TRY_CUDA(cudaLaunchKernelEx(&cfg, tpanel_kernel, W, ldw, mp, jb, ipiv, col0, info, kind, aop, aop_lo, R, plan,
                                   track, give_up, err));
  return 0;
}

// The panel's interchanges on all other columns, U12 = L11^-1 A12 on the
// right ones and their K-major B operand.  A warp per column.
template <typename T>
__global__ void __launch_bounds__(256)
sswap_trsm(T *W, int64_t ldw, int64_t n, int64_t j, int jb, const int32_t *plan, int kind, void *bop,
           float *bop_lo, int32_t *bexp, int64_t cap, const int32_t *abort) {
  if (abort != nullptr && *(volatile const int32_t *)abort != 0) return;  // set before this launch (same stream)
  __shared__ int32_t rows[2 * SNB], src[2 * SNB];
  __shared__ T L[SNB * SNB];
  __shared__ int cnt;
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
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= n - jb) return;
  const int64_t col = w < j ? w : w + jb;
  T *cp = W + col * ldw;
  T v[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) v[e] = lane + 32 * e < cnt ? cp[src[lane + 32 * e]] : T(0);
  __syncwarp();
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (lane + 32 * e < cnt) cp[rows[lane + 32 * e]] = v[e];
  __syncwarp();
  if (col < j + jb) return;
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

__global__ void zero_i32(int32_t *p) { *p = 0; }
__global__ void track_init(uint64_t *t) {
  t[0] = 0;                       // max |u_ii| = +0
  t[1] = 0x7ff0000000000000ull;   // min |u_ii| = +inf
  t[2] = 0;                       // not abandoned
}

template <typename P>
int launch_spanel(cudaStream_t s, typename P::G *W, int64_t ldw, int64_t mp, int jb, int32_t *ipiv, int32_t col0,
                  int32_t *info, int kind, void *aop, float *aop_lo, int32_t *aexp, int64_t cap, int32_t *plan,
                  uint64_t *track, double give_up, int32_t *err) {
  // FP64 panels are bound by the FP64 pipe of each CTA (~2 FMA per clock per
  // SM): short ones spread over up to 16 CTAs of more than 64 rows each
  const int C = (int)imin(SMAXC, imax(1, cdiv(mp, P::kFP64 ? 128 : SPT)));
  const int64_t R = cdiv(mp, C);
  const size_t smem = sizeof(typename P::S) * (size_t)jb * (size_t)panel_pitch<typename P::S>(R);
  if (smem > 200 * 1024) return fail(BOLA_ERR_UNSUPPORTED, "mixed LU: panel of %lld rows too tall", (long long)mp);
  static bool attr = false;
  if (!attr) {
    BOLA_TRY_CUDA(cudaFuncSetAttribute(spanel_kernel<P>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    BOLA_TRY_CUDA(cudaFuncSetAttribute(spanel_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C, 1, 1);
  cfg.blockDim = dim3(SPT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr1[1];
  attr1[0].id = cudaLaunchAttributeClusterDimension;
  attr1[0].val.clusterDim.x = (unsigned)C;
  attr1[0].val.clusterDim.y = 1;
  attr1[0].val.clusterDim.z = 1;
  cfg.attrs = attr1;
  cfg.numAttrs = 1;
  ProfScope prof(s, P::kFP64 ? "spanel64" : "spanel", (double)mp * jb * jb,
                 2.0 * sizeof(typename P::G) * (double)mp * jb);
  BOLA_TRY_CUDA(cudaLaunchKernelEx(&cfg, spanel_kernel<P>, W, ldw, mp, jb, ipiv, col0, info, kind, aop, aop_lo, aexp,
                                   cap, R, plan, track, give_up, err));
  return 0;
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
  BOLA_TRY_CUDA(cudaMallocAsync(&plan, sizeof(int32_t) * (1 + 4 * SNB), s));
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
                   reinterpret_cast<void **>(&ea[1]), reinterpret_cast<void **>(&eb)}) {
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

// Width of the panel starting at j: 64, or 48 for FP64 panels taller than
// the cluster's shared memory holds at 64 columns (16 x 399 rows).
int panel_width(bool fp64, int64_t n, int64_t j) {
  const int64_t mp = n - j;
  return (int)imin(fp64 && mp > SMAXC * 399 ? 48 : SNB, mp);
}

}  // namespace

// Right-looking blocked LU of W (n x n), ipiv global 1-based, *info the first
// zero pivot (the factor is then unusable; the caller falls back).  Kinds 0-2:
// FP32 W and tc_update; kind 3: FP64 W and the exact-split oz_update.  Per
// step k: panel, swaps + U12 + B operand, the update of the next panel's
// columns (all on sp), then the update of the other columns on su, which
// overlaps panel k+1; the swaps of step k+1 wait for it.
template <typename T>
static int factor_lookahead(MixedLU &lu, cudaStream_t s, T *W, int64_t ldw, int32_t *ipiv, int32_t *info,
                            double give_up) {
  constexpr bool fp64 = std::is_same<T, double>::value;
  const int64_t n = lu.n;
  BOLA_TRY_CUDA(cudaEventRecord(lu.ev_in, s));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.sp, lu.ev_in, 0));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.su, lu.ev_in, 0));
  zero_i32<<<1, 1, 0, lu.sp>>>(info);
  track_init<<<1, 1, 0, lu.sp>>>(lu.track);
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
    if constexpr (fp64)
      BOLA_TRY(launch_spanel<PanelF64>(lu.sp, W + j + j * ldw, ldw, mp, jb, ipiv + j, (int32_t)j, info, lu.kind,
                                       upd ? lu.aop[buf] : nullptr, nullptr, lu.ea[buf], lu.cap_n, lu.plan, track,
                                       give_up, lu.err));
    else
      BOLA_TRY(launch_tpanel(lu.sp, W + j + j * ldw, ldw, mp, jb, ipiv + j, (int32_t)j, info, lu.kind,
                             upd ? lu.aop[buf] : nullptr, lu.aop_lo[buf], lu.plan, track, give_up, lu.err));
    // the row swaps reach every column: the previous wide update must be done
    if (wide_pending) BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.sp, lu.ev_wide, 0));
    wide_pending = false;
    const int64_t others = n - jb;
    if (others > 0) {
      ProfScope prof(lu.sp, fp64 ? "sswap_trsm64" : "sswap_trsm", (double)jb * jb * (double)(n - j - jb));
      sswap_trsm<T><<<(unsigned)cdiv(others, 8), 256, 0, lu.sp>>>(W, ldw, n, j, jb, lu.plan, lu.kind,
                                                                    upd ? lu.bop : nullptr, fp64 ? nullptr : lu.bop_lo,
                                                                    fp64 ? lu.eb : nullptr, lu.cap_n, abort);
      BOLA_CHECK_LAUNCH();
    }
    if (!upd) continue;
    const int64_t m2 = mp - jb, n2 = n - j - jb;
    const int64_t nb_next = imin((int64_t)panel_width(fp64, n, j + jb), n2);
    T *W22 = W + (j + jb) + (j + jb) * ldw;
    auto update = [&](cudaStream_t st, int64_t cols, int64_t boff) -> int {
      if constexpr (fp64)
        return oz_update(st, m2, cols, lu.mapA[buf], lu.mapB, lu.cap_n, lu.cap_n, lu.ea[buf], lu.eb,
                         W22 + boff * ldw, ldw, lu.err, boff, abort);
      else
        return tc_update(st, lu.kind, m2, cols, lu.mapA[buf], lu.mapB, lu.mapAlo[buf], lu.mapBlo,
                         W22 + boff * ldw, ldw, lu.err, boff, abort);
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
  if (wide_pending) BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.sp, lu.ev_wide, 0));
  BOLA_TRY_CUDA(cudaEventRecord(lu.ev_done, lu.sp));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(s, lu.ev_done, 0));
  return 0;
}

int MixedLU::factor(cudaStream_t s, float *W, int64_t ldw, int32_t *ipiv, int32_t *info, double give_up) {
  return factor_lookahead<float>(*this, s, W, ldw, ipiv, info, give_up);
}

int MixedLU::factor64(cudaStream_t s, double *W, int64_t ldw, int32_t *ipiv, int32_t *info, double give_up) {
  return factor_lookahead<double>(*this, s, W, ldw, ipiv, info, give_up);
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
