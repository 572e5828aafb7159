// mixed.cuh — shared declarations of the mixed-precision solver's pieces.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace bola {

// Tensor map for a K-major operand buffer of `rows` rows x 64 K values
// (bf16 or fp32 elements), boxes of box_rows rows x 128 bytes, 128-byte swizzle.
int make_kmajor_map(CUtensorMap *map, const void *ptr, int64_t rows, bool bf16, int box_rows = 128);
// Tensor map for tiles of an FP64 column-major matrix (no swizzle).
int make_fp64_tile_map(CUtensorMap *map, const double *ptr, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                       int box_cols);

// ---- exact splitting of FP64 operands into bf16 slices (oz_update.cu) ----
// Row r of an operand with 64 K values v_k and exponent e (the largest
// |v_k| lies in [2^(e-1), 2^e)) is stored as OZ_SLICES bf16 integer slices,
// v_k = 2^(e-7) sum_t s_t,k 2^(-8t) (to within 2^(e-48)), slice t of row r at
// ((t*cap + r)*64 + k).  All of it is integer arithmetic: GB300's FP64 pipe is
// the scarce resource.
constexpr int OZ_SLICES = 6;

// |v| as ordered bits (sign cleared): the largest magnitude has the largest key.
__device__ __forceinline__ uint64_t oz_mag(double v) {
  return (uint64_t)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// e with the row's largest magnitude in [2^(e-1), 2^e), from oz_mag of it; 0 for a zero row.
__device__ __forceinline__ int oz_exponent(uint64_t mag_bits) {
  const int ev = (int)(mag_bits >> 52);
  return ev == 0 ? 0 : ev - 1022;
}

// The slices of v (|v| < 2^e) with integer operations only: X = round(v 2^(47-e))
// (|X| <= 2^47), then signed base-256 digits, least significant first, so that
// v ~ 2^(e-7) sum_t s_t 2^(-8t) with |s_t| <= 128.  Zeros and subnormals give 0.
__device__ __forceinline__ void oz_slices(double v, int e, __nv_bfloat16 (&s)[OZ_SLICES]) {
  const uint64_t bits = (uint64_t)__double_as_longlong(v);
  const int ev = (int)((bits >> 52) & 0x7FF);
  int64_t X = 0;
  if (ev != 0) {
    const uint64_t M = (bits & ((1ull << 52) - 1)) | (1ull << 52);  // v = M 2^(ev - 1075)
    const int k = 1028 - ev + e;                                    // >= 6 because |v| < 2^e
    if (k < 64) X = (int64_t)((M + (1ull << (k - 1))) >> k);
    if (bits >> 63) X = -X;
  }
#pragma unroll
  for (int t = OZ_SLICES - 1; t > 0; --t) {
    const int d = (int)((X + 128) & 255) - 128;
    s[t] = __int2bfloat16_rn(d);
    X = (X - d) >> 8;
  }
  s[0] = __int2bfloat16_rn((int)X);
}

// One row whose 64 K values a warp holds as (lane, lane + 32).
__device__ __forceinline__ void oz_split_pair(double v0, double v1, int lane, int64_t r, int64_t cap,
                                              __nv_bfloat16 *out, int32_t *ex) {
  uint64_t mb = oz_mag(v0) > oz_mag(v1) ? oz_mag(v0) : oz_mag(v1);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t o = __shfl_xor_sync(0xffffffffu, mb, off);
    mb = o > mb ? o : mb;
  }
  const int e = oz_exponent(mb);
  if (lane == 0) ex[r] = e;
  __nv_bfloat16 s0[OZ_SLICES], s1[OZ_SLICES];
  oz_slices(v0, e, s0);
  oz_slices(v1, e, s1);
#pragma unroll
  for (int t = 0; t < OZ_SLICES; ++t) {
    out[((int64_t)t * cap + r) * 64 + lane] = s0[t];
    out[((int64_t)t * cap + r) * 64 + lane + 32] = s1[t];
  }
}

// W(m x n, FP64) -= A B^T from the slices of A (rows of capA per slice) and
// B (capB), exponents eA[m], eB[n]; *err set if a bounded wait expired.
int oz_update(cudaStream_t s, int64_t m, int64_t n, const CUtensorMap &A, const CUtensorMap &B, int64_t capA,
              int64_t capB, const int32_t *eA, const int32_t *eB, double *W, int64_t ldw, int32_t *err,
              int64_t boff = 0, const int32_t *abort = nullptr);

// W(m x n, column-major, ld ldw) -= A * B^T on tcgen05 (kind 0 bf16, 1 tf32,
// 2 3xTF32 with the lo maps); *err is set non-zero if a bounded wait expired.
// B's rows start at boff (a column offset into the trailing matrix).
int tc_update(cudaStream_t s, int kind, int64_t m, int64_t n, const CUtensorMap &A, const CUtensorMap &B,
              const CUtensorMap &Alo, const CUtensorMap &Blo, float *W, int64_t ldw, int32_t *err, int64_t boff = 0,
              const int32_t *abort = nullptr);

// A kernel of an abandoned factorisation returns at once: *abort is read by
// one thread and the decision shared, so a CTA's barriers stay uniform even
// while another stream sets the flag.
__device__ __forceinline__ bool abandoned(const int32_t *abort) {
  __shared__ int skip;
  if (threadIdx.x == 0) skip = abort != nullptr && *(volatile const int32_t *)abort != 0;
  __syncthreads();
  return skip != 0;
}

// Buffers and tensor maps of the low-precision LU (slu.cu), reusable across
// factorisations of size <= capacity.  The factorisation looks ahead: the
// trailing update of step k is split into the next panel's columns (on the
// high-priority stream sp, with the panels and swaps) and the rest (on the
// low-priority stream su), so that panel k+1 runs on its cluster while the
// wide update of step k fills the other SMs.  The A operand is therefore
// double-buffered by step parity.
struct MixedLU {
  int64_t n = 0, cap_n = 0;
  int kind = -1;  // 0 bf16, 1 tf32, 2 3xTF32 update operands (FP32 W); 3 exact bf16 slices (FP64 W)
  void *aop[2] = {nullptr, nullptr}, *bop = nullptr;
  float *aop_lo[2] = {nullptr, nullptr}, *bop_lo = nullptr;
  int32_t *ea[2] = {nullptr, nullptr}, *eb = nullptr;  // kind 3: row exponents of the sliced operands
  int32_t *err = nullptr;
  int32_t *plan = nullptr;  // the current panel's composed interchanges: count, rows[128], src[128]
  // running extent of |u_ii| over the panels done: [0] max, [1] min (bits of
  // non-negative doubles, ordered like the values), [2] low word = abandon flag
  uint64_t *track = nullptr;
  CUtensorMap mapA[2], mapB, mapAlo[2], mapBlo;
  cudaStream_t sp = nullptr, su = nullptr;
  cudaEvent_t ev_in = nullptr, ev_sw = nullptr, ev_wide = nullptr, ev_done = nullptr;
  int reserve(int64_t n, int kind, cudaStream_t s);
  void release(cudaStream_t s);  // frees the buffers (stream-ordered on s)
  void destroy();                // the streams and events too (device idle)
  // LU with partial pivoting of the FP32 matrix W (n x n, ld ldw) in place (kinds 0-2).
  // give_up: the factorisation is abandoned (its kernels return at once) as
  // soon as max|u_ii| / min|u_ii| over the pivots so far is not below it;
  // INFINITY never gives up.  abandoned() on the host tells afterwards.
  int factor(cudaStream_t s, float *W, int64_t ldw, int32_t *ipiv, int32_t *info, double give_up = INFINITY);
  // The same for an FP64 W (kind 3).
  int factor64(cudaStream_t s, double *W, int64_t ldw, int32_t *ipiv, int32_t *info, double give_up = INFINITY);
};

}  // namespace bola
