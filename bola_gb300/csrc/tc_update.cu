// tc_update.cu — rank-64 update of an FP32 matrix on the 5th-generation
// tensor cores: W(m x n, column-major) -= A * B^T, A (m x 64) and B (n x 64)
// stored K-major (64 contiguous K values per row).
//
// This is the trailing update of the mixed-precision LU.  Operand forms:
//   kind 0: A, B bf16                (kind::f16, 4 MMAs of K=16)
//   kind 1: A, B tf32 (fp32 storage) (kind::tf32, 8 MMAs of K=8)
//   kind 2: 3xTF32: A = Ahi + Alo, B = Bhi + Blo, each term tf32-exact;
//           Ahi*Bhi + Ahi*Blo + Alo*Bhi accumulated in FP32 (~2^-22 accuracy)
// The update is HBM-bound: W is read and written once per step, while the MMA
// work per tile is ~0.1 us.  Two kernels:
//   tc_update_pipe   (W's leading dimension a multiple of 4, origin 16-byte
//                    aligned: every call of the factorisations) — a CTA runs
//                    through several 128x64 tiles with TMA loads, the MMA
//                    chain and the drain of consecutive tiles overlapped
//                    (warp-specialised, two TMEM accumulators, W moved by
//                    TMA through shared memory);
//   tc_update_kernel (any W) — one 128x128 tile per CTA, load, MMA and drain
//                    in sequence, W read and written by the drain warps.
#include <mutex>

#include "common.cuh"
#include "mixed.cuh"
#include "sm100.cuh"

namespace bola {
namespace {

using namespace sm100;

constexpr int BM = 128, BN = 128, KDIM = 64;
constexpr int BOX_BYTES = 128 * 128;  // one 128-row x 128-byte operand box

template <int KIND, int NPASS>
struct TcCfg {
  static constexpr int KB = KIND == 0 ? 1 : 2;           // 128-byte K boxes per operand for K = 64
  static constexpr int NOPS = NPASS == 3 ? 2 : 1;        // hi (and lo) copies
  static constexpr int TILE_BYTES = NOPS * KB * BOX_BYTES;  // per operand
  static constexpr int SMEM = 2 * TILE_BYTES + 1024;     // A + B + alignment slack
  // at most four CTAs per SM: four 128-column accumulators fill TMEM
  static constexpr int SMEM_LAUNCH = SMEM < 56 * 1024 ? 56 * 1024 : SMEM;
  static constexpr uint32_t IDESC = make_idesc(KIND == 0 ? 1u : 2u, BM, BN);
};

template <int KIND, int NPASS>
__global__ void __launch_bounds__(128)
tc_update_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                 const __grid_constant__ CUtensorMap mapAlo, const __grid_constant__ CUtensorMap mapBlo, int64_t m,
                 int64_t n, int64_t boff, float *__restrict__ W, int64_t ldw, int32_t *err, const int32_t *abort,
                 int lower) {
  using Cfg = TcCfg<KIND, NPASS>;
  // a Cholesky update leaves the tiles strictly above the diagonal alone
  if (lower && boff + (int64_t)blockIdx.y * BN >= (int64_t)blockIdx.x * BM + BM) return;
  if (abandoned(abort)) return;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_slot;
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *tileA = base;
  uint8_t *tileB = base + Cfg::TILE_BYTES;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t i0 = (int64_t)blockIdx.x * BM, j0 = (int64_t)blockIdx.y * BN;

  if (tid == 0) {
    mbar_init(&bar_load, 1);
    mbar_init(&bar_mma, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(&tmem_slot, 128);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  __shared__ int ok_shared;
  if (tid == 0) {
    ok_shared = 1;
    mbar_arrive_expect_tx(&bar_load, 2 * Cfg::TILE_BYTES);
    for (int op = 0; op < Cfg::NOPS; ++op) {
      for (int kb = 0; kb < Cfg::KB; ++kb) {
        const int x = kb * (KIND == 0 ? 64 : 32);
        tma_load_2d(tileA + (op * Cfg::KB + kb) * BOX_BYTES, op ? &mapAlo : &mapA, x, (int32_t)i0, &bar_load);
        // B's maps have 64-row boxes (shared with the pipelined kernel): two per tile
        tma_load_2d(tileB + (op * Cfg::KB + kb) * BOX_BYTES, op ? &mapBlo : &mapB, x, (int32_t)(boff + j0),
                    &bar_load);
        tma_load_2d(tileB + (op * Cfg::KB + kb) * BOX_BYTES + BOX_BYTES / 2, op ? &mapBlo : &mapB, x,
                    (int32_t)(boff + j0 + 64), &bar_load);
      }
    }
    if (!bounded_wait(&bar_load, 0)) {
      ok_shared = 0;
      atomicExch(err, 1);
    } else {
      tc_fence_after();
      uint32_t acc = 0;
      constexpr int NP = NPASS;
      for (int p = 0; p < NP; ++p) {
        const int aop = (p == 2) ? 1 : 0;  // passes: (hi,hi), (hi,lo), (lo,hi)
        const int bop = (p == 1) ? 1 : 0;
        for (int kb = 0; kb < Cfg::KB; ++kb) {
          const uint64_t da = sw128_kmajor_desc(tileA + (aop * Cfg::KB + kb) * BOX_BYTES);
          const uint64_t db = sw128_kmajor_desc(tileB + (bop * Cfg::KB + kb) * BOX_BYTES);
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {  // 4 MMAs per 128-byte row: K = 16 (bf16) or 8 (tf32)
            umma<KIND == 0 ? 0 : 1>(tmem, desc_advance(da, ks * 32), desc_advance(db, ks * 32), Cfg::IDESC, acc);
            acc = 1;
          }
        }
      }
      umma_commit(&bar_mma);
    }
  }
  __syncthreads();
  const bool ok = ok_shared != 0;
  if (ok) {
    if (!bounded_wait(&bar_mma, 0)) {
      atomicExch(err, 2);
    } else {
      tc_fence_after();
      const int64_t row = i0 + warp * 32 + lane;
      float *wrow = W + row + j0 * ldw;
      const int64_t ncols = n - j0 < BN ? n - j0 : BN;
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        // issue the 32 loads of W first so they are all in flight together
        float w[32];
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) {
          const int cc = c * 32 + jj;
          w[jj] = (row < m && cc < ncols) ? __ldcs(wrow + cc * ldw) : 0.f;
        }
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
        if (row < m) {
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) {
            const int cc = c * 32 + jj;
            if (cc < ncols) __stcs(wrow + cc * ldw, w[jj] - v[jj]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

// ---- the pipelined form ------------------------------------------------------------
// Each CTA runs through a short range of consecutive 128 x 64 tiles (the same
// rows of A for most of them): warp 0 streams A (once per row block), B and
// the FP32 tile of W itself through TMA into a resident A buffer and
// two-stage B and W rings; warp 1 issues the MMA chain into one of two
// 64-column TMEM accumulators; eight epilogue warps subtract the other
// accumulator from its W tile in shared memory, and one thread stores the tile
// back with TMA.  Load, MMA and drain of consecutive tiles overlap, so a tile
// costs about its W traffic (read + write, 64 KB) instead of the sum of the
// three phases.  The range is kept short (TPC tiles) so that CTAs come and go
// like single-tile CTAs: the factorisation's panel, launched on a
// higher-priority stream while a wide update runs, still finds free SMs.
constexpr int PBN = 64;    // tile columns
constexpr int PEPI = 8;    // epilogue warps
constexpr int PTHREADS = 64 + 32 * PEPI;

template <int KIND, int NPASS>
struct PCfg {
  static constexpr int KB = KIND == 0 ? 1 : 2;  // 128-byte K boxes per row for K = 64
  static constexpr int NOPS = NPASS == 3 ? 2 : 1;
  static constexpr int A_BYTES = NOPS * KB * BM * 128;
  static constexpr int B_BYTES = NOPS * KB * PBN * 128;
  static constexpr int W_BYTES = BM * PBN * 4;
  static constexpr int SMEM = A_BYTES + 2 * B_BYTES + 2 * W_BYTES + 1024;
  static constexpr uint32_t IDESC = make_idesc(KIND == 0 ? 1u : 2u, BM, PBN);
};

__device__ __forceinline__ void bulk_wait_all0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Named barrier over the epilogue warps that also ORs a per-thread flag: every
// warp leaves with the same answer, so all of them stop on the same tile.
__device__ __forceinline__ bool epilogue_bar_any(bool flag) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"((uint32_t)flag), "r"(32 * PEPI)
      : "memory");
  return r != 0;
}

// The next tile at or after linear index T (row-block-major, NT tiles per row
// block) that a lower (Cholesky) update keeps; t1 if none before it.
__device__ __forceinline__ int next_tile(int T, int t1, int NT, int64_t boff, bool lower) {
  for (; T < t1; ++T) {
    const int i = T / NT, j = T % NT;
    if (!lower || boff + (int64_t)j * PBN < (int64_t)i * BM + BM) return T;
  }
  return t1;
}

template <int KIND, int NPASS>
__global__ void __launch_bounds__(PTHREADS, 1)
tc_update_pipe(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
               const __grid_constant__ CUtensorMap mapAlo, const __grid_constant__ CUtensorMap mapBlo,
               const __grid_constant__ CUtensorMap mapW, const __grid_constant__ CUtensorMap mapWs, int64_t m,
               int64_t n, int64_t boff, int tpc, int32_t *err, const int32_t *abort, int lower, float *W,
               int64_t ldw) {
  using Cfg = PCfg<KIND, NPASS>;
  sm100::grid_dependency_wait();
  if (abandoned(abort)) return;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t a_full, a_empty, b_full[2], b_empty[2], w_full[2], w_empty[2], acc_full[2], acc_empty[2];
  __shared__ uint32_t tmem_slot;
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *tileA = base;
  uint8_t *tileB = base + Cfg::A_BYTES;                           // two stages
  float *tileW = reinterpret_cast<float *>(tileB + 2 * Cfg::B_BYTES);  // two stages, [64 columns][128 rows]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int NT = (int)cdiv(n, PBN), MT = (int)cdiv(m, BM);
  const int t0 = blockIdx.x * tpc, t1 = (int)imin((int64_t)MT * NT, (int64_t)t0 + tpc);
  const bool low = lower != 0;

  if (tid == 0) {
    mbar_init(&a_full, 1);
    mbar_init(&a_empty, 1);
    for (int q = 0; q < 2; ++q) {
      mbar_init(&b_full[q], 1);
      mbar_init(&b_empty[q], 1);
      mbar_init(&w_full[q], 1);
      mbar_init(&w_empty[q], 1);
      mbar_init(&acc_full[q], 1);
      mbar_init(&acc_empty[q], PEPI);
    }
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(&tmem_slot, 2 * PBN);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // -- producer
      int k = 0, ai = -1, na = 0;
      for (int T = next_tile(t0, t1, NT, boff, low); T < t1; T = next_tile(T + 1, t1, NT, boff, low), ++k) {
        const int i = T / NT, j = T % NT;
        if (i != ai) {
          if (na > 0 && !bounded_wait(&a_empty, (uint32_t)(na - 1) & 1u)) {
            atomicExch(err, 21);
            break;
          }
          mbar_arrive_expect_tx(&a_full, Cfg::A_BYTES);
          for (int op = 0; op < Cfg::NOPS; ++op)
            for (int kb = 0; kb < Cfg::KB; ++kb)
              tma_load_2d(tileA + (op * Cfg::KB + kb) * BM * 128, op ? &mapAlo : &mapA, kb * (KIND == 0 ? 64 : 32),
                          i * BM, &a_full);
          ai = i;
          ++na;
        }
        const int st = k & 1;
        const uint32_t ph = (uint32_t)(k >> 1) & 1u;
        if (!bounded_wait(&b_empty[st], ph ^ 1u) || !bounded_wait(&w_empty[st], ph ^ 1u)) {
          atomicExch(err, 22);
          break;
        }
        mbar_arrive_expect_tx(&b_full[st], Cfg::B_BYTES);
        for (int op = 0; op < Cfg::NOPS; ++op)
          for (int kb = 0; kb < Cfg::KB; ++kb)
            tma_load_2d(tileB + st * Cfg::B_BYTES + (op * Cfg::KB + kb) * PBN * 128, op ? &mapBlo : &mapB,
                        kb * (KIND == 0 ? 64 : 32), (int32_t)(boff + (int64_t)j * PBN), &b_full[st]);
        mbar_arrive_expect_tx(&w_full[st], Cfg::W_BYTES);
        tma_load_2d(tileW + st * (BM * PBN), &mapW, i * BM, j * PBN, &w_full[st]);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // -- MMA issuer
      int k = 0, ai = -1, na = 0;
      for (int T = next_tile(t0, t1, NT, boff, low); T < t1; ++k) {
        const int i = T / NT;
        const int Tn = next_tile(T + 1, t1, NT, boff, low);
        if (i != ai) {
          if (!bounded_wait(&a_full, (uint32_t)na & 1u)) {
            atomicExch(err, 23);
            break;
          }
          ai = i;
          ++na;
        }
        const int st = k & 1;
        const uint32_t ph = (uint32_t)(k >> 1) & 1u;
        if (!bounded_wait(&b_full[st], ph) || !bounded_wait(&acc_empty[st], ph ^ 1u)) {
          atomicExch(err, 24);
          break;
        }
        tc_fence_after();
        uint32_t acc = 0;
        for (int p = 0; p < NPASS; ++p) {
          const int aop = (p == 2) ? 1 : 0;  // passes: (hi,hi), (hi,lo), (lo,hi)
          const int bop = (p == 1) ? 1 : 0;
          for (int kb = 0; kb < Cfg::KB; ++kb) {
            const uint64_t da = sw128_kmajor_desc(tileA + (aop * Cfg::KB + kb) * BM * 128);
            const uint64_t db = sw128_kmajor_desc(tileB + st * Cfg::B_BYTES + (bop * Cfg::KB + kb) * PBN * 128);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              umma<KIND == 0 ? 0 : 1>(tmem + (uint32_t)(st * PBN), desc_advance(da, ks * 32),
                                      desc_advance(db, ks * 32), Cfg::IDESC, acc);
              acc = 1;
            }
          }
        }
        umma_commit(&b_empty[st]);
        umma_commit(&acc_full[st]);
        if (Tn >= t1 || Tn / NT != i) umma_commit(&a_empty);  // the next tile loads other rows of A
        T = Tn;
      }
    }
  } else {
    // -- epilogue: warp w drains TMEM lanes 32 (w % 4).. (its tile rows), columns 32 h ..
    const int ew = warp - 2, q = warp & 3, h = ew >> 2;
    const int r = q * 32 + lane;
    int k = 0;
    for (int T = next_tile(t0, t1, NT, boff, low); T < t1; T = next_tile(T + 1, t1, NT, boff, low), ++k) {
      const int i = T / NT, j = T % NT;
      const int st = k & 1;
      const uint32_t ph = (uint32_t)(k >> 1) & 1u;
      // a wait that expires is reported, and every epilogue warp still meets
      // the barrier below before all of them leave together
      const bool ok = __all_sync(0xffffffffu, bounded_wait(&acc_full[st], ph) && bounded_wait(&w_full[st], ph));
      if (!ok && lane == 0) atomicExch(err, 25);
      float *Ws = tileW + st * (BM * PBN);
      if (ok) {
        tc_fence_after();
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(st * PBN + h * 32), v);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[st]);
#pragma unroll
        for (int c = 0; c < 32; ++c) Ws[(h * 32 + c) * BM + r] -= v[c];
        // the last 1-3 rows when m is not a multiple of 4: the tile store
        // (mapWs) covers m & ~3 rows only — a TMA store clips the innermost
        // dimension at 16-byte granularity, and the rows past m belong to the
        // caller (ldw > m) — so these go by plain stores
        const int64_t row = (int64_t)i * BM + r;
        if (row >= (m & ~(int64_t)3) && row < m) {
          for (int c = 0; c < 32; ++c) {
            const int64_t col = (int64_t)j * PBN + h * 32 + c;
            if (col < n) W[row + col * ldw] = Ws[(h * 32 + c) * BM + r];
          }
        }
      }
      fence_proxy_async_smem();
      if (epilogue_bar_any(!ok)) break;  // the epilogue warps only
      if (ew == 0 && lane == 0) {
        tma_store_2d(&mapWs, Ws, i * BM, j * PBN);  // rows (past m & ~3) and columns outside W are clipped
        bulk_commit();
        bulk_wait_read0();
        mbar_arrive(&w_empty[st]);
      }
    }
    if (ew == 0 && lane == 0) bulk_wait_all0();  // the stores have landed before the CTA ends
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, 2 * PBN);
}

// ---- host: tensor maps ----------------------------------------------------------
using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  });
  return fn;
}

}  // namespace

// K-major operand: `rows` rows of 64 K values (bf16: 128 B per row; fp32: 256 B), boxes of box_rows rows.
int make_kmajor_map(CUtensorMap *map, const void *ptr, int64_t rows, bool bf16, int box_rows) {
  EncodeFn enc = encode_fn();
  if (!enc) return fail(BOLA_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[2] = {(cuuint64_t)KDIM, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)KDIM * (bf16 ? 2 : 4)};
  const cuuint32_t box[2] = {bf16 ? 64u : 32u, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                         const_cast<void *>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(BOLA_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return 0;
}

int make_kmajor_map2(CUtensorMap *map, const void *ptr, int64_t kdim, int64_t rows, int64_t kp, int box_rows) {
  EncodeFn enc = encode_fn();
  if (!enc) return fail(BOLA_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[2] = {(cuuint64_t)kdim, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
  const cuuint32_t box[2] = {64u, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(BOLA_ERR_CUDA, "cuTensorMapEncodeTiled (digit planes) failed (%d)", (int)r);
  return 0;
}

// FP64 column-major matrix (rows x cols, ld), boxes of box_rows x box_cols,
// no swizzle (ld * 8 and the origin must be multiples of 16 bytes).
int make_fp64_tile_map(CUtensorMap *map, const double *ptr, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                       int box_cols) {
  EncodeFn enc = encode_fn();
  if (!enc) return fail(BOLA_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 8};
  const cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double *>(ptr), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(BOLA_ERR_CUDA, "cuTensorMapEncodeTiled (fp64 tile) failed (%d)", (int)r);
  return 0;
}

// FP32 column-major matrix (rows x cols, ld), boxes of 128 rows x 64
// columns, no swizzle (ld * 4 and the origin must be multiples of 16 bytes).
int make_fp32_tile_map(CUtensorMap *map, const float *ptr, int64_t rows, int64_t cols, int64_t ld) {
  EncodeFn enc = encode_fn();
  if (!enc) return fail(BOLA_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
  const cuuint32_t box[2] = {(cuuint32_t)BM, (cuuint32_t)PBN};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(ptr), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(BOLA_ERR_CUDA, "cuTensorMapEncodeTiled (fp32 tile) failed (%d)", (int)r);
  return 0;
}

int tc_update(cudaStream_t s, int kind, int64_t m, int64_t n, const CUtensorMap &A, const CUtensorMap &B,
              const CUtensorMap &Alo, const CUtensorMap &Blo, float *W, int64_t ldw, int32_t *err, int64_t boff,
              const int32_t *abort, bool lower, bool pdl) {
  if (m <= 0 || n <= 0) return 0;
  ProfScope prof(s, "tc_update", 2.0 * (double)m * n * KDIM * (kind == 2 ? 3 : 1), 8.0 * (double)m * n);
  if ((ldw & 3) == 0 && (reinterpret_cast<uintptr_t>(W) & 15) == 0 && m >= 4) {
    // the pipelined kernel: W's tiles move by TMA (16-byte aligned rows);
    // loads see all m rows, the tile store m & ~3 of them (the rest are
    // stored by the epilogue threads)
    CUtensorMap mapW, mapWs;
    BOLA_TRY(make_fp32_tile_map(&mapW, W, m, n, ldw));
    BOLA_TRY(make_fp32_tile_map(&mapWs, W, m & ~(int64_t)3, n, ldw));
    const int64_t tiles = cdiv(m, BM) * cdiv(n, PBN);
    // runs of up to 8 tiles per CTA, but never fewer CTAs than twice the SMs
    // (a narrow update, on the critical path, keeps one tile per CTA)
    const int tpc = (int)imax(1, imin(8, tiles / (2 * (int64_t)num_sms())));
    const unsigned grid = (unsigned)cdiv(tiles, tpc);
#define BOLA_TCP(KIND, NPASS)                                                                                   \
  do {                                                                                                          \
    using Cfg = PCfg<KIND, NPASS>;                                                                              \
    static bool attr = false;                                                                                   \
    if (!attr) {                                                                                                \
      BOLA_TRY_CUDA(                                                                                            \
          cudaFuncSetAttribute(tc_update_pipe<KIND, NPASS>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM)); \
      attr = true;                                                                                              \
    }                                                                                                           \
    StepLaunch L(dim3(grid), dim3(PTHREADS), Cfg::SMEM, s, pdl);                                                \
    BOLA_TRY_CUDA(cudaLaunchKernelEx(&L.cfg, tc_update_pipe<KIND, NPASS>, A, B, Alo, Blo, mapW, mapWs, m, n, boff,  \
                                     tpc, err, abort, lower ? 1 : 0, W, ldw));                                  \
  } while (0)
    if (kind == 0) BOLA_TCP(0, 1);
    else if (kind == 1) BOLA_TCP(1, 1);
    else BOLA_TCP(1, 3);
#undef BOLA_TCP
    BOLA_CHECK_LAUNCH();
    return 0;
  }
  const dim3 grid((unsigned)cdiv(m, BM), (unsigned)cdiv(n, BN));
#define BOLA_TC(KIND, NPASS)                                                                              \
  do {                                                                                                    \
    using Cfg = TcCfg<KIND, NPASS>;                                                                       \
    static bool attr = false;                                                                             \
    if (!attr) {                                                                                          \
      BOLA_TRY_CUDA(cudaFuncSetAttribute(tc_update_kernel<KIND, NPASS>,                                   \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM_LAUNCH)); \
      attr = true;                                                                                        \
    }                                                                                                     \
    tc_update_kernel<KIND, NPASS><<<grid, 128, Cfg::SMEM_LAUNCH, s>>>(A, B, Alo, Blo, m, n, boff, W, ldw, err, abort, lower ? 1 : 0); \
  } while (0)
  if (kind == 0) BOLA_TC(0, 1);
  else if (kind == 1) BOLA_TC(1, 1);
  else BOLA_TC(1, 3);
#undef BOLA_TC
  BOLA_CHECK_LAUNCH();
  return 0;
}

}  // namespace bola

extern "C" int bola_sgemm_tc_update(int kind, int64_t m, int64_t n, const void *a, const void *b, const void *a_lo,
                                    const void *b_lo, float *w, int64_t ldw, int32_t *err, bola_stream_t stream) {
  using namespace bola;
  if (kind < 0 || kind > 2) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (ldw < imax(1, m)) return -9;
  if (m == 0 || n == 0) return 0;
  const bool bf16 = kind == 0;
  CUtensorMap A, B, Alo, Blo;
  BOLA_TRY(make_kmajor_map(&A, a, m, bf16));
  BOLA_TRY(make_kmajor_map(&B, b, n, bf16, 64));
  BOLA_TRY(make_kmajor_map(&Alo, kind == 2 ? a_lo : a, m, bf16));
  BOLA_TRY(make_kmajor_map(&Blo, kind == 2 ? b_lo : b, n, bf16, 64));
  return tc_update((cudaStream_t)stream, kind, m, n, A, B, Alo, Blo, w, ldw, err, 0);
}
