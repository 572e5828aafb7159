// oz_update.cu — FP64-accurate rank-64 update on the bf16 tensor cores
// (no BOLA counterpart; the trailing update of the FP64-storage mixed LU).
//
//   W(m x n, FP64, column-major) -= A B^T,   A: m x 64, B: n x 64 (FP64)
//
// by exact splitting (the Ozaki scheme): every row of A (and of B) is scaled
// by a power of two so that its largest entry lies in [64, 128) and then cut
// into OZ_SLICES integer slices of at most 8 bits each,
//   a_k = 2^(e-7) * sum_t s_t,k 2^(-8t),   |s_t,k| <= 128,
// stored as bf16 (exact for integers up to 256).  A product of two slices is
// an integer below 2^14 in magnitude, a K = 64 sum of them stays below 2^20,
// and adding the (at most OZ_SLICES) slice pairs of equal weight t + u = d
// stays below 2^23: every partial sum the tensor core forms in its FP32
// accumulator is an integer under 2^24, so the accumulation is exact
// whatever its order.  Pairs of weight d <= OZ_DMAX = 6 are kept (26 of the
// 36); the dropped pairs and the slicing remainder each stay near
// 2^-48 * 64 * max|a_i.| * max|b_j.|, so the result is FP64-accurate relative
// to the scales of the rows involved.  The epilogue combines the OZ_DMAX + 1
// accumulators, W -= 2^(eA + eB - 14) * sum_d 2^(-8d) acc_d, on the integer
// pipe: GB300 retires only about two FP64 operations per clock per SM, so
// the exact accumulators become one 64-bit fixed-point sum (unit 2^-40),
// which integer bit operations turn into a double; the subtraction from W is
// the only FP64 instruction per element.
//
// Per CTA: a 128 x 64 tile of W.  A's slices (128 rows) and B's (64 rows)
// arrive by TMA with 128-byte swizzle, and the FP64 tile of W itself by TMA
// too (64 KB, in flight while the MMAs run); one thread issues the 26 x 4
// tcgen05.mma (kind::f16, M = 128, N = 64, K = 16) into seven 64-column TMEM
// accumulators; eight warps drain them with tcgen05.ld (warps w and w + 4
// share TMEM lanes 32(w%4).. and split the 64 columns), update the W tile in
// shared memory, and one TMA store writes it back.  W's leading dimension
// must be even and its tile origins 16-byte aligned (TMA).
#include <cuda_bf16.h>

#include "common.cuh"
#include "mixed.cuh"
#include "sm100.cuh"

namespace bola {
namespace {

using namespace sm100;

constexpr int OBM = 128, OBN = 64, OK = 64;
constexpr int S = OZ_SLICES;
constexpr int DMAX = 6;  // highest pair weight t + u kept
constexpr int NPAIRS = 26;
constexpr int A_BOX = OBM * 128;  // bytes of one A slice tile (128 rows x 64 bf16)
constexpr int B_BOX = OBN * 128;  // bytes of one B slice tile
constexpr int W_BOX = OBM * OBN * 8;  // the FP64 tile of W, column-major 128 x 64
constexpr int OZ_SMEM = S * (A_BOX + B_BOX) + W_BOX + 1024;
constexpr uint32_t OZ_IDESC = make_idesc(1u, OBM, OBN);
constexpr int OZ_TMEM_COLS = 512;  // (DMAX + 1) * 64 = 448 columns used

// T * 2^E as a double, T a 64-bit integer, rounded to nearest (ties away
// from zero) with integer operations only; ldexp for results outside the
// normal range.
__device__ __forceinline__ double fix_to_double(int64_t T, int E) {
  if (T == 0) return 0.0;
  const bool neg = T < 0;
  uint64_t a = neg ? (uint64_t)(-T) : (uint64_t)T;
  const int lz = __clzll((long long)a);
  a <<= lz;                                   // leading one at bit 63
  uint64_t m = (a >> 11) + ((a >> 10) & 1u);  // 53 significant bits, rounded
  int e = 63 - lz;                            // T = a * 2^(e - 63)
  if (m >> 53) {
    m >>= 1;
    e += 1;
  }
  const int field = 1023 + e + E;
  if (field <= 0 || field >= 2047) return ldexp((double)T, E);
  const uint64_t bits = ((uint64_t)neg << 63) | ((uint64_t)field << 52) | (m & ((1ull << 52) - 1));
  return __longlong_as_double((long long)bits);
}

// 32 lanes x 16 consecutive 32-bit TMEM columns.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

constexpr int OZ_THREADS = 256;

__global__ void __launch_bounds__(OZ_THREADS)
oz_update_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                 const __grid_constant__ CUtensorMap mapW, int64_t capA, int64_t capB, int64_t boff, int64_t m,
                 int64_t n, const int32_t *__restrict__ eA, const int32_t *__restrict__ eB, int32_t *err,
                 const int32_t *abort, int lower) {
  // a Cholesky update leaves the tiles strictly above the diagonal alone
  if (lower && boff + (int64_t)blockIdx.y * OBN >= (int64_t)blockIdx.x * OBM + OBM) return;
  if (abandoned(abort)) return;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_slot;
  __shared__ int ok_shared;
  __shared__ int32_t ebs[OBN];
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *tileA = base;                // S tiles of A_BOX bytes
  uint8_t *tileB = base + S * A_BOX;    // S tiles of B_BOX bytes
  double *tileW = reinterpret_cast<double *>(base + S * (A_BOX + B_BOX));  // [64 columns][128 rows]

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t i0 = (int64_t)blockIdx.x * OBM, j0 = (int64_t)blockIdx.y * OBN;

  if (tid == 0) {
    mbar_init(&bar_load, 1);
    mbar_init(&bar_mma, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(&tmem_slot, OZ_TMEM_COLS);
    tmem_relinquish();
  }
  if (tid < OBN) ebs[tid] = j0 + tid < n ? eB[boff + j0 + tid] : 0;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (tid == 0) {
    ok_shared = 1;
    mbar_arrive_expect_tx(&bar_load, S * (A_BOX + B_BOX) + W_BOX);
    tma_load_2d(tileW, &mapW, (int32_t)i0, (int32_t)j0, &bar_load);
    for (int t = 0; t < S; ++t) {
      tma_load_2d(tileA + t * A_BOX, &mapA, 0, (int32_t)(t * capA + i0), &bar_load);
      tma_load_2d(tileB + t * B_BOX, &mapB, 0, (int32_t)(t * capB + boff + j0), &bar_load);
    }
    if (!bounded_wait(&bar_load, 0)) {
      ok_shared = 0;
      atomicExch(err, 1);
    } else {
      tc_fence_after();
      for (int d = 0; d <= DMAX; ++d) {  // accumulator d collects the pairs t + u = d
        const uint32_t acc_addr = tmem + (uint32_t)(d * OBN);
        uint32_t acc = 0;
        for (int t = (d > S - 1 ? d - (S - 1) : 0); t <= d && t < S; ++t) {
          const int u = d - t;
          const uint64_t da = sw128_kmajor_desc(tileA + t * A_BOX);
          const uint64_t db = sw128_kmajor_desc(tileB + u * B_BOX);
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {  // K = 64 as 4 x 16 bf16 (32 bytes each)
            umma<0>(acc_addr, desc_advance(da, ks * 32), desc_advance(db, ks * 32), OZ_IDESC, acc);
            acc = 1;
          }
        }
      }
      umma_commit(&bar_mma);
    }
  }
  __syncthreads();
  if (ok_shared != 0) {
    if (!bounded_wait(&bar_mma, 0)) {
      atomicExch(err, 2);
    } else {
      tc_fence_after();
      const int rl = (warp & 3) * 32 + lane;
      const int64_t row = i0 + rl;
      const int ea = row < m ? eA[row] : 0;
      const int cbeg = (warp >> 2) * (OBN / 2);
#pragma unroll 1
      for (int c0 = cbeg; c0 < cbeg + OBN / 2; c0 += 16) {
        // sum_d acc_d 2^(-8d) in units of 2^-40: |acc_0| <= 2^20, so |T| < 2^61
        int64_t T[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) T[q] = 0;
#pragma unroll
        for (int d = 0; d <= DMAX; ++d) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(d * OBN + c0), v);
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int64_t iv = (int64_t)__float2int_rn(v[q]);  // exact: |acc_d| < 2^23
            T[q] += d <= 5 ? (iv << (8 * (5 - d))) : (iv >> (8 * (d - 5)));
          }
        }
        // rows and columns outside W are clipped by the TMA store
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          double *p = tileW + (c0 + q) * OBM + rl;
          *p -= fix_to_double(T[q], ea + ebs[c0 + q] - 54);
        }
      }
      fence_proxy_async_smem();
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && ok_shared != 0) {
    tma_store_2d(&mapW, tileW, (int32_t)i0, (int32_t)j0);
    bulk_commit();
    bulk_wait_read0();
  }
  if (warp == 0) tmem_dealloc(tmem, OZ_TMEM_COLS);
}

// Slices of rows of an FP64 K-major matrix (rows x 64, ld 64): one warp per
// row, two K values per lane.
__global__ void oz_split_rows(int64_t rows, const double *__restrict__ X, int64_t cap, __nv_bfloat16 *out,
                              int32_t *ex) {
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  const double v0 = X[r * OK + lane], v1 = X[r * OK + lane + 32];
  oz_split_pair(v0, v1, lane, r, cap, out, ex);
}

}  // namespace

int oz_update(cudaStream_t s, int64_t m, int64_t n, const CUtensorMap &A, const CUtensorMap &B, int64_t capA,
              int64_t capB, const int32_t *eA, const int32_t *eB, double *W, int64_t ldw, int32_t *err, int64_t boff,
              const int32_t *abort, bool lower) {
  if (m <= 0 || n <= 0) return 0;
  if ((ldw & 1) != 0 || (reinterpret_cast<uintptr_t>(W) & 15) != 0)
    return fail(BOLA_ERR_UNSUPPORTED, "oz_update: W needs an even leading dimension and a 16-byte aligned origin");
  CUtensorMap mapW;
  BOLA_TRY(make_fp64_tile_map(&mapW, W, m, n, ldw, OBM, OBN));
  static bool attr = false;
  if (!attr) {
    BOLA_TRY_CUDA(cudaFuncSetAttribute(oz_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM));
    attr = true;
  }
  const dim3 grid((unsigned)cdiv(m, OBM), (unsigned)cdiv(n, OBN));
  ProfScope prof(s, "oz_update", 2.0 * (double)m * n * OK * NPAIRS, 16.0 * (double)m * n);
  oz_update_kernel<<<grid, OZ_THREADS, OZ_SMEM, s>>>(A, B, mapW, capA, capB, boff, m, n, eA, eB, err, abort,
                                                     lower ? 1 : 0);
  BOLA_CHECK_LAUNCH();
  return 0;
}

}  // namespace bola

extern "C" int bola_dgemm_oz_update(int64_t m, int64_t n, const double *a, const double *b, double *w, int64_t ldw,
                                    int32_t *err, bola_stream_t stream) {
  using namespace bola;
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldw < imax(1, m)) return -6;
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  __nv_bfloat16 *sa = nullptr, *sb = nullptr;
  int32_t *ea = nullptr, *eb = nullptr;
  BOLA_TRY_CUDA(cudaMallocAsync(&sa, sizeof(__nv_bfloat16) * S * m * OK, s));
  BOLA_TRY_CUDA(cudaMallocAsync(&sb, sizeof(__nv_bfloat16) * S * n * OK, s));
  BOLA_TRY_CUDA(cudaMallocAsync(&ea, sizeof(int32_t) * m, s));
  BOLA_TRY_CUDA(cudaMallocAsync(&eb, sizeof(int32_t) * n, s));
  oz_split_rows<<<(unsigned)cdiv(m, 8), 256, 0, s>>>(m, a, m, sa, ea);
  oz_split_rows<<<(unsigned)cdiv(n, 8), 256, 0, s>>>(n, b, n, sb, eb);
  CUtensorMap A, B;
  int st = make_kmajor_map(&A, sa, S * m, true, OBM);
  if (st == 0) st = make_kmajor_map(&B, sb, S * n, true, OBN);
  if (st == 0) st = oz_update(s, m, n, A, B, m, n, ea, eb, w, ldw, err, 0);
  for (void *p : {(void *)sa, (void *)sb, (void *)ea, (void *)eb}) cudaFreeAsync(p, s);
  return st;
}
