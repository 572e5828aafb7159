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
// converted to a double once and scaled through its exponent field; the
// subtraction from W is the only FP64 arithmetic per element.
//
// Tiles of W are 128 x 64.  A's slices (128 rows) and B's (64 rows) arrive
// by TMA with 128-byte swizzle; one thread issues the 26 x 4 tcgen05.mma
// (kind::f16, M = 128, N = 64, K = 16) into seven 64-column TMEM
// accumulators, one per weight; sixteen warps drain them with tcgen05.ld
// (the four warps with the same w % 4 share TMEM lanes 32(w%4).. and split
// the 64 columns) and update W in place.  Warp-specialised and pipelined across the tiles a
// CTA runs through (oz_update_pipe below).
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
constexpr uint32_t OZ_IDESC = make_idesc(1u, OBM, OBN);
constexpr int OZ_TMEM_COLS = 512;  // (DMAX + 1) * 64 = 448 columns used

// T * 2^E as a double, T a 64-bit integer: one conversion (rounded to
// nearest even), then the power of two added to the exponent field when the
// result stays normal (exact); ldexp otherwise.
__device__ __forceinline__ double fix_to_double(int64_t T, int E) {
  const double x = (double)T;
  const long long b = __double_as_longlong(x);
  const int field = (int)((b >> 52) & 0x7FF) + E;
  if (T == 0) return 0.0;
  if (field <= 0 || field >= 2047) return ldexp(x, E);
  return __longlong_as_double(b + ((long long)E << 52));
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

// ---- the update kernel ---------------------------------------------------------------
// Each CTA runs through a short range of consecutive 128 x 64 tiles of W
// (row-block-major, so most of them share A's rows).  Warp 0 streams A's
// slices (once per row block, resident) and B's (a two-stage ring) through
// TMA, and prefetches the tile of W into L2; warp 1 issues the MMA chains and
// commits each weight's accumulator on its own mbarrier; sixteen epilogue warps
// drain accumulator d as soon as its pairs are done and hand it back, so the
// next tile's MMAs for weight d start while the epilogue still reads weights
// d + 1 ... of this one.  The drain is a chain of dependent integer steps per
// element, so it takes sixteen warps (four per SM sub-partition, 16 columns
// each) to keep the sub-partitions issuing.  W is read and written directly by
// the epilogue (a warp moves 32 consecutive rows of a column per access),
// which keeps shared memory to A's and B's slices.  The accumulators combine into three 32-bit
// partial sums (weights 0-1, 2-3 and 4-6) before the 64-bit fixed-point sum:
// the same integer as adding every weight into 64 bits.
constexpr int ZEPI = 16;                   // epilogue warps: four per TMEM lane quadrant
constexpr int ZCOL = OBN / (ZEPI / 4);     // columns an epilogue warp drains
constexpr int ZTHREADS = 64 + 32 * ZEPI;   // producer warp, MMA warp, epilogue
constexpr int ZA_BYTES = S * A_BOX;        // A's slices of one row block
constexpr int ZB_BYTES = S * B_BOX;        // B's slices of one tile (one ring stage)
constexpr int ZSMEM = ZA_BYTES + 2 * ZB_BYTES + 1024;

// The next tile at or after linear index T (row-block-major, NT tiles per row
// block) that a lower (Cholesky) update keeps; t1 if none before it.
__device__ __forceinline__ int oz_next_tile(int T, int t1, int NT, int64_t boff, bool lower) {
  for (; T < t1; ++T) {
    const int i = T / NT, j = T % NT;
    if (!lower || boff + (int64_t)j * OBN < (int64_t)i * OBM + OBM) return T;
  }
  return t1;
}

// An integer-valued float v with |v| <= 2^22, as an int (an FP32 add and an
// integer subtract instead of a conversion instruction).
__device__ __forceinline__ int small_int(float v) { return __float_as_int(v + 12582912.0f) - 0x4B400000; }

__global__ void __launch_bounds__(ZTHREADS, 1)
oz_update_pipe(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int64_t capA,
               int64_t capB, int64_t boff, int64_t m, int64_t n, const int32_t *__restrict__ eA,
               const int32_t *__restrict__ eB, double *__restrict__ W, int64_t ldw, int tpc, int32_t *err,
               const int32_t *abort, int lower) {
  sm100::grid_dependency_wait();
  if (abandoned(abort)) return;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t a_full, a_empty, b_full[2], b_empty[2], acc_full[DMAX + 1], acc_empty[DMAX + 1];
  __shared__ uint32_t tmem_slot;
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *tileA = base;             // S slices of A_BOX bytes
  uint8_t *tileB = base + ZA_BYTES;  // two stages of S slices of B_BOX bytes
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int NT = (int)cdiv(n, OBN), MT = (int)cdiv(m, OBM);
  const int t0 = blockIdx.x * tpc, t1 = (int)imin((int64_t)MT * NT, (int64_t)t0 + tpc);
  const bool low = lower != 0;
  // bulk prefetches need 16-byte aligned column starts
  const bool wpre = (ldw & 1) == 0 && (reinterpret_cast<uintptr_t>(W) & 15) == 0;

  if (tid == 0) {
    mbar_init(&a_full, 1);
    mbar_init(&a_empty, 1);
    for (int q = 0; q < 2; ++q) {
      mbar_init(&b_full[q], 1);
      mbar_init(&b_empty[q], 1);
    }
    for (int d = 0; d <= DMAX; ++d) {
      mbar_init(&acc_full[d], 1);
      mbar_init(&acc_empty[d], ZEPI);
    }
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(&tmem_slot, OZ_TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // -- producer
      int k = 0, ai = -1, na = 0;
      for (int T = oz_next_tile(t0, t1, NT, boff, low); T < t1; T = oz_next_tile(T + 1, t1, NT, boff, low), ++k) {
        const int i = T / NT, j = T % NT;
        if (i != ai) {
          if (na > 0 && !bounded_wait(&a_empty, (uint32_t)(na - 1) & 1u)) {
            atomicExch(err, 31);
            break;
          }
          mbar_arrive_expect_tx(&a_full, ZA_BYTES);
          for (int t = 0; t < S; ++t)
            tma_load_2d(tileA + t * A_BOX, &mapA, 0, (int32_t)(t * capA + (int64_t)i * OBM), &a_full);
          ai = i;
          ++na;
        }
        const int st = k & 1;
        if (!bounded_wait(&b_empty[st], ((uint32_t)(k >> 1) & 1u) ^ 1u)) {
          atomicExch(err, 32);
          break;
        }
        mbar_arrive_expect_tx(&b_full[st], ZB_BYTES);
        for (int u = 0; u < S; ++u)
          tma_load_2d(tileB + st * ZB_BYTES + u * B_BOX, &mapB, 0, (int32_t)(u * capB + boff + (int64_t)j * OBN),
                      &b_full[st]);
        if (wpre) {  // W's tile into L2 ahead of the epilogue: one bulk prefetch per column
          const int64_t r0 = (int64_t)i * OBM, cb = (int64_t)j * OBN;
          const uint32_t bytes = (uint32_t)(imin(OBM, m - r0) * 8) & ~15u;
          const int nc = (int)imin(OBN, n - cb);
          if (bytes > 0)
            for (int c = 0; c < nc; ++c) bulk_prefetch_l2(W + r0 + (cb + c) * ldw, bytes);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // -- MMA issuer
      int k = 0, ai = -1, na = 0;
      bool ok = true;
      for (int T = oz_next_tile(t0, t1, NT, boff, low); T < t1 && ok; ++k) {
        const int i = T / NT;
        const int Tn = oz_next_tile(T + 1, t1, NT, boff, low);
        if (i != ai) {
          if (!bounded_wait(&a_full, (uint32_t)na & 1u)) {
            atomicExch(err, 33);
            break;
          }
          ai = i;
          ++na;
        }
        const int st = k & 1;
        if (!bounded_wait(&b_full[st], (uint32_t)(k >> 1) & 1u)) {
          atomicExch(err, 34);
          break;
        }
        for (int d = 0; d <= DMAX; ++d) {  // accumulator d collects the pairs t + u = d
          // the epilogue has read this accumulator for the previous tile
          if (!bounded_wait(&acc_empty[d], ((uint32_t)k & 1u) ^ 1u)) {
            atomicExch(err, 35);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t acc_addr = tmem + (uint32_t)(d * OBN);
          uint32_t acc = 0;
          for (int t = (d > S - 1 ? d - (S - 1) : 0); t <= d && t < S; ++t) {
            const uint64_t da = sw128_kmajor_desc(tileA + t * A_BOX);
            const uint64_t db = sw128_kmajor_desc(tileB + st * ZB_BYTES + (d - t) * B_BOX);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {  // K = 64 as 4 x 16 bf16 (32 bytes each)
              umma<0>(acc_addr, desc_advance(da, ks * 32), desc_advance(db, ks * 32), OZ_IDESC, acc);
              acc = 1;
            }
          }
          umma_commit(&acc_full[d]);
        }
        if (!ok) break;
        umma_commit(&b_empty[st]);
        if (Tn >= t1 || Tn / NT != i) umma_commit(&a_empty);  // the next tile loads other rows of A
        T = Tn;
      }
    }
  } else {
    // -- epilogue: warp w drains TMEM lanes 32 (w % 4).. (its tile rows), columns ZCOL h ..
    const int ew = warp - 2, q = warp & 3, h = ew >> 2;
    const int rl = q * 32 + lane;
    int k = 0;
    for (int T = oz_next_tile(t0, t1, NT, boff, low); T < t1; T = oz_next_tile(T + 1, t1, NT, boff, low), ++k) {
      const int i = T / NT, j = T % NT;
      const int64_t row = (int64_t)i * OBM + rl;
      const int64_t c0 = (int64_t)j * OBN + h * ZCOL;  // this warp's first column
      const int ncol = (int)imax(0, imin(ZCOL, n - c0));
      int Z[ZCOL], Y[ZCOL], X[ZCOL];  // weights 0-1, 2-3, 4-6 (the partial sums below)
      bool ok = true;
#pragma unroll
      for (int d = 0; d <= DMAX; ++d) {
        ok = ok && __all_sync(0xffffffffu, bounded_wait(&acc_full[d], (uint32_t)k & 1u));
        if (ok) tc_fence_after();
        const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(d * OBN + h * ZCOL);
#pragma unroll
        for (int hb = 0; hb < ZCOL; hb += 16) {
          float v[16];
          if (ok) {
            tmem_ld16(ta + hb, v);
          } else {
#pragma unroll
            for (int c = 0; c < 16; ++c) v[c] = 0.f;
          }
          // |acc_d| <= (pairs of weight d) * 64 * 2^14: <= 2^22 for d <= 3
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const int cc = hb + c;
            if (d == 0) Z[cc] = small_int(v[c]);
            if (d == 1) Z[cc] = Z[cc] * 256 + small_int(v[c]);  // |Z| <= 2^28 + 2^21
            if (d == 2) Y[cc] = small_int(v[c]);
            if (d == 3) Y[cc] = Y[cc] * 256 + small_int(v[c]);  // |Y| <= 3 * 2^28 + 2^22
            if (d == 4) X[cc] = __float2int_rn(v[c]);            // <= 5 * 2^20
            if (d == 5) X[cc] = X[cc] * 256 + __float2int_rn(v[c]);
            if (d == 6) X[cc] += __float2int_rn(v[c]) >> 8;      // |X| < 1.26 * 2^30
          }
        }
        if (ok) {  // the accumulator goes back to the MMA issuer
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&acc_empty[d]);
        }
      }
      if (!ok) {
        if (lane == 0) atomicExch(err, 36);
        break;
      }
      if (row < m) {
        double *wp = W + row + c0 * ldw;  // (prefetched into L2 by the producer)
        const int ea = eA[row];
        const int32_t *eb = eB + boff + c0;
        double x[ZCOL];
#pragma unroll
        for (int c = 0; c < ZCOL; ++c) {
          // sum_d acc_d 2^(-8d) in units of 2^-40
          const int64_t Tq = ((int64_t)Z[c] << 32) + ((int64_t)Y[c] << 16) + (int64_t)X[c];
          x[c] = c < ncol ? fix_to_double(Tq, ea + eb[c] - 54) : 0.0;
        }
        // all of W's loads first (no store between them), then the stores
        double w[ZCOL];
#pragma unroll
        for (int c = 0; c < ZCOL; ++c) w[c] = c < ncol ? wp[c * ldw] : 0.0;
#pragma unroll
        for (int c = 0; c < ZCOL; ++c)
          if (c < ncol) wp[c * ldw] = w[c] - x[c];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, OZ_TMEM_COLS);
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
              const int32_t *abort, bool lower, bool pdl) {
  if (m <= 0 || n <= 0) return 0;
  static bool attr = false;
  if (!attr) {
    BOLA_TRY_CUDA(cudaFuncSetAttribute(oz_update_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize, ZSMEM));
    attr = true;
  }
  const int64_t tiles = cdiv(m, OBM) * cdiv(n, OBN);
  // runs of up to 8 tiles per CTA, but never fewer CTAs than twice the SMs
  // (a narrow update, on the critical path, keeps one tile per CTA)
  const int tpc = (int)imax(1, imin(8, tiles / (2 * (int64_t)num_sms())));
  const unsigned grid = (unsigned)cdiv(tiles, tpc);
  ProfScope prof(s, "oz_update", 2.0 * (double)m * n * OK * NPAIRS, 16.0 * (double)m * n);
  StepLaunch L(dim3(grid), dim3(ZTHREADS), ZSMEM, s, pdl);
  BOLA_TRY_CUDA(cudaLaunchKernelEx(&L.cfg, oz_update_pipe, A, B, capA, capB, boff, m, n, eA, eB, W, ldw, tpc, err,
                                   abort, lower ? 1 : 0));
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
