// slu.cu — the low-precision LU of the mixed-precision solver (no BOLA
// counterpart; it preconditions the FP64 refinement in ir.cu).
//
// A (FP64) is scaled per 64-column block by a power of two (exact) and
// rounded to an FP32 working matrix W.  Blocked right-looking LU with partial
// pivoting and NB = 64 = the K of the tensor-core update:
//   spanel_kernel   the (n-j) x 64 panel on a cluster of <=16 CTAs, the rows
//                   held in shared memory; per column each CTA pushes its pivot
//                   candidate (key + row) into every CTA's shared memory, so
//                   a column costs one CTA barrier pair and one cluster
//                   barrier.  It also writes L21 as the K-major A operand
//                   (bf16, or tf32 hi/lo) of the update.
//   sswap_trsm      the 64 interchanges on every other column, U12 = L11^-1 A12
//                   and the K-major B operand.
//   tc_update       W22 -= L21 U12 on tcgen05 with FP32 accumulation in TMEM.
// Pivots are this algorithm's own; only the FP64 refinement decides accuracy.
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "mixed.cuh"

namespace cg = cooperative_groups;

namespace bola {
namespace {

constexpr int SNB = 64;   // panel width and update depth
constexpr int SPT = 256;  // threads per panel CTA
constexpr int SMAXC = 16;

struct SSlot {
  uint32_t khi, klo;  // |pivot candidate| bits, ~row
  float v[SNB];       // the candidate row
};

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t u = __float_as_uint(x);
  u = (u + 0x1000u) & ~0x1FFFu;
  return __uint_as_float(u);
}

// Writes one 64-wide row of an update operand (K-major, row `r`).
__device__ __forceinline__ void write_operand_row(int kind, void *op, float *op_lo, int64_t r, const float *v) {
  if (kind == 0) {
    __nv_bfloat16 *d = static_cast<__nv_bfloat16 *>(op) + r * SNB;
#pragma unroll
    for (int c = 0; c < SNB; c += 8) {
      __align__(16) __nv_bfloat16 t[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) t[u] = __float2bfloat16_rn(v[c + u]);
      *reinterpret_cast<uint4 *>(d + c) = *reinterpret_cast<const uint4 *>(t);
    }
  } else {
    float *d = static_cast<float *>(op) + r * SNB;
    float *dl = op_lo + r * SNB;
#pragma unroll
    for (int c = 0; c < SNB; c += 4) {
      float4 h, l;
      h.x = tf32_round(v[c]);
      h.y = tf32_round(v[c + 1]);
      h.z = tf32_round(v[c + 2]);
      h.w = tf32_round(v[c + 3]);
      *reinterpret_cast<float4 *>(d + c) = h;
      if (kind == 2) {
        l.x = tf32_round(v[c] - h.x);
        l.y = tf32_round(v[c + 1] - h.y);
        l.z = tf32_round(v[c + 2] - h.z);
        l.w = tf32_round(v[c + 3] - h.w);
        *reinterpret_cast<float4 *>(dl + c) = l;
      }
    }
  }
}

// Panel LU of W[0:mp, 0:jb] (W points at the panel's top-left).  ipiv gets
// global 1-based rows (col0 + local + 1).  CTA cr of the cluster owns panel
// rows [cr*R, cr*R + R), kept in shared memory column-major with an odd
// pitch (R + 1) so that both a thread walking its row and a warp walking a
// column are conflict-free.
//
// Per column j: pivot search in column j, one CTA barrier, every warp pushes
// the CTA's candidate row (and row j if the CTA owns it) into its share of
// the CTAs, cluster-barrier ARRIVE; then, while the other CTAs catch up, the
// rank-1 update of pivot j-1 on columns j+1.. (deferred from the previous
// column); cluster-barrier WAIT; every CTA picks the same winner from its own
// slots and brings the pushed rows up to date (they left before pivot j-1's
// deferred update reached their columns > j: the same fmaf the owner does);
// swap; one CTA barrier; the update of column j+1 only (the next pivot
// column).  Multipliers of column j are scaled when column j+1 is searched.
__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(SPT)
spanel_kernel(float *W, int64_t ldw, int64_t mp, int jb, int32_t *ipiv, int32_t col0, int32_t *info, int kind,
              void *aop, float *aop_lo, int64_t R, int32_t *plan) {
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int cr = (int)cluster.block_rank();
  __shared__ SSlot slots[2][SMAXC];
  __shared__ float rowj[2][SNB];
  __shared__ float piv[2][SNB];   // pivot rows, up to date (piv[par] = column j's)
  __shared__ float oldj[SNB];     // the old row j, up to date (goes to the pivot's place)
  __shared__ uint64_t wkey[SPT / 32];
  extern __shared__ float sp[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int RP = (int)R + 1;
  const int r0 = (int)(cr * R);
  const int r1 = (int)imin(mp, r0 + R);
  const int nr = r1 > r0 ? r1 - r0 : 0;

  for (int64_t e = tid; e < (int64_t)nr * jb; e += SPT) {
    const int il = (int)(e % nr);
    const int c = (int)(e / nr);
    sp[c * RP + il] = W[(r0 + il) + c * ldw];
  }
  __syncthreads();
  cluster.sync();  // every CTA of the cluster is running before the first push

  float inv = 0.f;  // 1 / pivot of the previous column
  for (int j = 0; j < jb; ++j) {
    const int par = j & 1;
    const float *pprev = piv[par ^ 1];
    // -- the multipliers of column j-1, then this CTA's pivot candidate in
    // column j: key = (|v| bits, ~row), max wins, ties -> lowest row
    uint64_t best = 0;
    for (int il = tid; il < nr; il += SPT) {
      const int g = r0 + il;
      if (j > 0 && g >= j) sp[(j - 1) * RP + il] *= inv;
      if (g < j) continue;
      const float v = fabsf(sp[j * RP + il]);
      const uint32_t bits = (v == v) ? __float_as_uint(v) : 0u;
      const uint64_t key = ((uint64_t)bits << 32) | (0xFFFFFFFFu - (uint32_t)g);
      best = key > best ? key : best;
    }
    const uint32_t hi = (uint32_t)(best >> 32), lo = (uint32_t)best;
    const uint32_t mhi = __reduce_max_sync(0xffffffffu, hi);
    const uint32_t mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
    if (lane == 0) wkey[warp] = ((uint64_t)mhi << 32) | mlo;
    __syncthreads();
    // -- every warp pushes the candidate (and row j if owned) to its share of the CTAs
    {
      uint64_t ck = 0;
#pragma unroll
      for (int w = 0; w < SPT / 32; ++w) ck = wkey[w] > ck ? wkey[w] : ck;
      const int gl = ck ? (int)(0xFFFFFFFFu - (uint32_t)ck) - r0 : -1;  // local row of the candidate
      const bool own_j = j >= r0 && j < r1;
      const int jl = j - r0;
      float c0 = 0.f, c1 = 0.f, j0v = 0.f, j1v = 0.f;
      if (gl >= 0) {
        c0 = lane < jb ? sp[lane * RP + gl] : 0.f;
        c1 = lane + 32 < jb ? sp[(lane + 32) * RP + gl] : 0.f;
      }
      if (own_j) {
        j0v = lane < jb ? sp[lane * RP + jl] : 0.f;
        j1v = lane + 32 < jb ? sp[(lane + 32) * RP + jl] : 0.f;
      }
      for (int d = warp; d < C; d += SPT / 32) {
        SSlot *rs = cluster.map_shared_rank(&slots[par][cr], d);
        if (lane == 0) {
          rs->khi = (uint32_t)(ck >> 32);
          rs->klo = (uint32_t)ck;
        }
        rs->v[lane] = c0;
        rs->v[lane + 32] = c1;
        if (own_j) {
          float *rj = cluster.map_shared_rank(&rowj[par][0], d);
          rj[lane] = j0v;
          rj[lane + 32] = j1v;
        }
      }
    }
    __syncthreads();  // the rows are read before the deferred update changes them
    cluster_arrive();
    // -- the deferred rank-1 update of pivot j-1 on columns j+1..jb-1, rows >= j:
    // lanes walk rows, warps take every 8th column; the pivot-row values sit
    // in registers, so a thread's 8 loads are all in flight together
    if (j > 0 && j + 1 < jb) {
      float pr[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int c = j + 1 + warp + 8 * q;
        pr[q] = c < jb ? pprev[c] : 0.f;
      }
      const int ib = j > r0 ? j - r0 : 0;
      for (int il = ib + lane; il < nr; il += 32) {
        const float l = sp[(j - 1) * RP + il];
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int c = j + 1 + warp + 8 * q;
          v[q] = c < jb ? sp[c * RP + il] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = fmaf(-l, pr[q], v[q]);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int c = j + 1 + warp + 8 * q;
          if (c < jb) sp[c * RP + il] = v[q];
        }
      }
    }
    cluster_wait();
    // -- the winner, identical in every CTA: lane s reads slot s, warp max
    uint64_t wk = 0;
    {
      const uint64_t k = lane < C ? (((uint64_t)slots[par][lane].khi << 32) | slots[par][lane].klo) : 0ull;
      const uint32_t khi = (uint32_t)(k >> 32);
      const uint32_t mh = __reduce_max_sync(0xffffffffu, khi);
      const uint32_t ml = __reduce_max_sync(0xffffffffu, khi == mh ? (uint32_t)k : 0u);
      wk = ((uint64_t)mh << 32) | ml;
    }
    int ws = 0;
    {
      const uint64_t k = lane < C ? (((uint64_t)slots[par][lane].khi << 32) | slots[par][lane].klo) : 0ull;
      const unsigned m = __ballot_sync(0xffffffffu, k == wk && lane < C);
      ws = m ? __ffs(m) - 1 : 0;
    }
    const int jp = wk ? (int)(0xFFFFFFFFu - (uint32_t)wk) : j;
    const float *raw = wk ? slots[par][ws].v : rowj[par];
    float *pcur = piv[par];
    // the pushed rows, brought up to date: columns > j still lack pivot j-1
    if (tid < jb) {
      float pv_ = raw[tid], ov = rowj[par][tid];
      if (j > 0 && tid > j) {
        pv_ = fmaf(-raw[j - 1], pprev[tid], pv_);
        ov = fmaf(-rowj[par][j - 1], pprev[tid], ov);
      }
      pcur[tid] = pv_;
      oldj[tid] = ov;
    }
    __syncthreads();
    const float pv = pcur[j];
    if (cr == 0 && tid == 0) ipiv[j] = col0 + jp + 1;
    inv = 1.0f / pv;
    if (pv == 0.0f) {
      inv = 0.0f;
      if (cr == 0 && tid == 0) atomicCAS(info, 0, col0 + j + 1);
    }
    if (jp != j && tid < jb) {
      if (j >= r0 && j < r1) sp[tid * RP + (j - r0)] = pcur[tid];
      if (jp >= r0 && jp < r1) sp[tid * RP + (jp - r0)] = oldj[tid];
    }
    __syncthreads();
    // -- the next pivot column now (the rest of this update is deferred);
    // same row-to-thread map as the search, so no barrier before it
    if (j + 1 < jb) {
      const float pj1 = pcur[j + 1];
      for (int il = tid; il < nr; il += SPT) {
        if (r0 + il <= j) continue;
        float *x = sp + (j + 1) * RP + il;
        *x = fmaf(-(sp[j * RP + il] * inv), pj1, *x);
      }
    }
  }
  // the last column's multipliers
  for (int il = tid; il < nr; il += SPT)
    if (r0 + il >= jb) sp[(jb - 1) * RP + il] *= inv;
  __syncthreads();

  // -- write back the panel and the update's A operand (rows below the panel)
  for (int64_t e = tid; e < (int64_t)nr * jb; e += SPT) {
    const int il = (int)(e % nr);
    const int c = (int)(e / nr);
    W[(r0 + il) + c * ldw] = sp[c * RP + il];
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
      float v[SNB];
#pragma unroll
      for (int c = 0; c < SNB; ++c) v[c] = c < jb ? sp[c * RP + il] : 0.f;
      write_operand_row(kind, aop, aop_lo, g - jb, v);
    }
  }
  cluster.sync();
}

// The panel's interchanges on all other columns, U12 = L11^-1 A12 on the
// right ones and their K-major B operand.  A warp per column.
__global__ void __launch_bounds__(256)
sswap_trsm(float *W, int64_t ldw, int64_t n, int64_t j, int jb, const int32_t *plan, int kind, void *bop,
           float *bop_lo) {
  __shared__ int32_t rows[2 * SNB], src[2 * SNB];
  __shared__ float L[SNB * SNB];
  __shared__ int cnt;
  // the interchanges, composed once by the panel kernel
  if (threadIdx.x == 0) cnt = plan[0];
  for (int t = threadIdx.x; t < 2 * SNB; t += blockDim.x) {
    rows[t] = plan[1 + t];
    src[t] = plan[1 + 2 * SNB + t];
  }
  for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) {
    const int r = e % jb, c = e / jb;
    L[r + c * SNB] = W[(j + r) + (j + c) * ldw];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= n - jb) return;
  const int64_t col = w < j ? w : w + jb;
  float *cp = W + col * ldw;
  float v[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) v[e] = lane + 32 * e < cnt ? cp[src[lane + 32 * e]] : 0.f;
  __syncwarp();
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (lane + 32 * e < cnt) cp[rows[lane + 32 * e]] = v[e];
  __syncwarp();
  if (col < j + jb) return;
  float b0 = lane < jb ? cp[j + lane] : 0.f;
  float b1 = lane + 32 < jb ? cp[j + lane + 32] : 0.f;
  for (int k = 0; k < jb; ++k) {
    const float bk = __shfl_sync(0xffffffffu, k < 32 ? b0 : b1, k & 31);
    if (lane > k) b0 = fmaf(-L[lane + k * SNB], bk, b0);
    if (lane + 32 > k && lane + 32 < jb) b1 = fmaf(-L[lane + 32 + k * SNB], bk, b1);
  }
  if (lane < jb) cp[j + lane] = b0;
  if (lane + 32 < jb) cp[j + lane + 32] = b1;
  if (bop != nullptr) {
    // row (col - j - jb) of the K-major B operand: the 64 values of U12's column
    __shared__ float stage[8][SNB];
    float *st = stage[threadIdx.x >> 5];
    st[lane] = lane < jb ? b0 : 0.f;
    st[lane + 32] = lane + 32 < jb ? b1 : 0.f;
    __syncwarp();
    if (lane == 0) write_operand_row(kind, bop, bop_lo, col - j - jb, st);
  }
}

__global__ void zero_i32(int32_t *p) { *p = 0; }

int launch_spanel(cudaStream_t s, float *W, int64_t ldw, int64_t mp, int jb, int32_t *ipiv, int32_t col0,
                  int32_t *info, int kind, void *aop, float *aop_lo, int32_t *plan) {
  const int C = (int)imin(SMAXC, imax(1, cdiv(mp, SPT)));
  const int64_t R = cdiv(mp, C);
  const size_t smem = sizeof(float) * SNB * (size_t)(R + 1);
  if (smem > 200 * 1024) return fail(BOLA_ERR_UNSUPPORTED, "mixed LU: panel of %lld rows too tall", (long long)mp);
  static bool attr = false;
  if (!attr) {
    BOLA_TRY_CUDA(cudaFuncSetAttribute(spanel_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    BOLA_TRY_CUDA(cudaFuncSetAttribute(spanel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
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
  ProfScope prof(s, "spanel", (double)mp * SNB * SNB, 8.0 * (double)mp * SNB);
  BOLA_TRY_CUDA(cudaLaunchKernelEx(&cfg, spanel_kernel, W, ldw, mp, jb, ipiv, col0, info, kind, aop, aop_lo, R, plan));
  return 0;
}

}  // namespace

int MixedLU::reserve(int64_t n_, int kind_, cudaStream_t s) {
  if (n_ <= cap_n && kind_ == kind && aop) {
    n = n_;
    return 0;
  }
  release(s);
  n = cap_n = n_;
  kind = kind_;
  const size_t esz = kind == 0 ? 2 : 4;
  BOLA_TRY_CUDA(cudaMallocAsync(&aop, (size_t)n * SNB * esz, s));
  BOLA_TRY_CUDA(cudaMallocAsync(&bop, (size_t)n * SNB * esz, s));
  if (kind == 2) {
    BOLA_TRY_CUDA(cudaMallocAsync(&aop_lo, (size_t)n * SNB * 4, s));
    BOLA_TRY_CUDA(cudaMallocAsync(&bop_lo, (size_t)n * SNB * 4, s));
  }
  BOLA_TRY_CUDA(cudaMallocAsync(&err, sizeof(int32_t), s));
  BOLA_TRY_CUDA(cudaMallocAsync(&plan, sizeof(int32_t) * (1 + 4 * SNB), s));
  BOLA_TRY_CUDA(cudaMemsetAsync(err, 0, sizeof(int32_t), s));
  const bool bf = kind == 0;
  BOLA_TRY(make_kmajor_map(&mapA, aop, n, bf));
  BOLA_TRY(make_kmajor_map(&mapB, bop, n, bf));
  BOLA_TRY(make_kmajor_map(&mapAlo, kind == 2 ? aop_lo : aop, n, bf));
  BOLA_TRY(make_kmajor_map(&mapBlo, kind == 2 ? bop_lo : bop, n, bf));
  return 0;
}

void MixedLU::release(cudaStream_t s) {
  for (void **p : {&aop, &bop, reinterpret_cast<void **>(&aop_lo), reinterpret_cast<void **>(&bop_lo),
                   reinterpret_cast<void **>(&err), reinterpret_cast<void **>(&plan)}) {
    if (*p) cudaFreeAsync(*p, s);
    *p = nullptr;
  }
  cap_n = 0;
}

// Right-looking blocked LU of W (n x n FP32), ipiv global 1-based, *info the
// first zero pivot (the factor is then unusable; the caller falls back).
int MixedLU::factor(cudaStream_t s, float *W, int64_t ldw, int32_t *ipiv, int32_t *info) {
  zero_i32<<<1, 1, 0, s>>>(info);
  BOLA_CHECK_LAUNCH();
  for (int64_t j = 0; j < n; j += SNB) {
    const int jb = (int)imin(SNB, n - j);
    const int64_t mp = n - j;
    const bool upd = j + jb < n;
    BOLA_TRY(launch_spanel(s, W + j + j * ldw, ldw, mp, jb, ipiv + j, (int32_t)j, info, kind, upd ? aop : nullptr,
                           aop_lo, plan));
    const int64_t others = n - jb;
    if (others > 0) {
      ProfScope prof(s, "sswap_trsm", (double)jb * jb * (double)(n - j - jb));
      sswap_trsm<<<(unsigned)cdiv(others, 8), 256, 0, s>>>(W, ldw, n, j, jb, plan, kind, upd ? bop : nullptr, bop_lo);
      BOLA_CHECK_LAUNCH();
    }
    if (upd) BOLA_TRY(tc_update(s, kind, mp - jb, n - j - jb, mapA, mapB, mapAlo, mapBlo,
                                W + (j + jb) + (j + jb) * ldw, ldw, err));
  }
  return 0;
}

}  // namespace bola
