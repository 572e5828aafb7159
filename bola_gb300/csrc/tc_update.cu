// tc_update.cu — rank-64 update of an FP32 matrix on the 5th-generation
// tensor cores: W(m x n, column-major) -= A * B^T, A (m x 64) and B (n x 64)
// stored K-major (64 contiguous K values per row).
//
// This is the trailing update of the mixed-precision LU: per 128x128 tile,
// one CTA loads its A and B tiles with TMA (128-byte swizzle), one thread
// issues the tcgen05.mma chain into a 128-column TMEM accumulator, and the
// four warps read the FP32 accumulator back with tcgen05.ld and subtract it
// from W in place.  Operand forms:
//   kind 0: A, B bf16                (kind::f16, 4 MMAs of K=16)
//   kind 1: A, B tf32 (fp32 storage) (kind::tf32, 8 MMAs of K=8)
//   kind 2: 3xTF32: A = Ahi + Alo, B = Bhi + Blo, each term tf32-exact;
//           Ahi*Bhi + Ahi*Blo + Alo*Bhi accumulated in FP32 (~2^-22 accuracy)
// The update is HBM-bound (W is read and written once per step; the MMA work
// per tile is ~0.1 us), so one tile per CTA and up to four CTAs per SM keep
// the memory system busy while each CTA's accumulator drains.
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
        tma_load_2d(tileB + (op * Cfg::KB + kb) * BOX_BYTES, op ? &mapBlo : &mapB, x, (int32_t)(boff + j0),
                    &bar_load);
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

int tc_update(cudaStream_t s, int kind, int64_t m, int64_t n, const CUtensorMap &A, const CUtensorMap &B,
              const CUtensorMap &Alo, const CUtensorMap &Blo, float *W, int64_t ldw, int32_t *err, int64_t boff,
              const int32_t *abort, bool lower) {
  if (m <= 0 || n <= 0) return 0;
  const dim3 grid((unsigned)cdiv(m, BM), (unsigned)cdiv(n, BN));
  ProfScope prof(s, "tc_update", 2.0 * (double)m * n * KDIM * (kind == 2 ? 3 : 1), 8.0 * (double)m * n);
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
  BOLA_TRY(make_kmajor_map(&B, b, n, bf16));
  BOLA_TRY(make_kmajor_map(&Alo, kind == 2 ? a_lo : a, m, bf16));
  BOLA_TRY(make_kmajor_map(&Blo, kind == 2 ? b_lo : b, n, bf16));
  return tc_update((cudaStream_t)stream, kind, m, n, A, B, Alo, Blo, w, ldw, err, 0);
}
