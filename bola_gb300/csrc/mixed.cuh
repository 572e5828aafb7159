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

// ---- FP64-accurate products A X on the tensor cores (oz_residual.cu) ----
// A is split once into OZ_SA digit planes (8-bit signed digits under a scale
// per row), X per product into OZ_SX planes (a scale per column); the planes
// pairs (t, u) with t + u <= OZ_D are accumulated exactly.
constexpr int OZ_SA = 7, OZ_SX = 8, OZ_D = 7;

// Tensor map for a row-major bf16 array with kdim K values per row (row pitch
// kp elements, a multiple of 64), `rows` rows, boxes of 64 K x box_rows rows,
// 128-byte swizzle; K beyond kdim reads as zero.
int make_kmajor_map2(CUtensorMap *map, const void *ptr, int64_t kdim, int64_t rows, int64_t kp, int box_rows);

struct OzMatrix {
  int64_t n = 0, cap = 0, mrows = 0, kp = 0, bytes = 0;
  bool ready = false;
  __nv_bfloat16 *planes = nullptr, *xplanes = nullptr;
  int32_t *e = nullptr, *f = nullptr;  // exponents of A's rows and of X's columns
  unsigned long long *rmax = nullptr, *acc = nullptr;
  double *psum = nullptr;
  CUtensorMap mapA, mapX;
  int reserve(int64_t n);
  void release();
  // A's digit planes; rowsum (optional, n doubles) gets sum_j |a_ij|
  int split(cudaStream_t s, const double *A, int64_t lda, double *rowsum);
  // out = b - A x (b != nullptr) or A x for nr columns; *err set if a bounded wait expired
  int product(cudaStream_t s, int nr, const double *x, int64_t ldx, const double *b, int64_t ldb, double *out,
              int64_t ldo, int32_t *err);
};

// Round to the nearest tf32 value (10 mantissa bits), ties away from zero.
__device__ __forceinline__ float tf32_round(float x) {
  uint32_t u = __float_as_uint(x);
  u = (u + 0x1000u) & ~0x1FFFu;
  return __uint_as_float(u);
}

// Writes one 64-wide row of an update operand (K-major, row `r`).
__device__ __forceinline__ void write_operand_row(int kind, void *op, float *op_lo, int64_t r, const float *v) {
  if (kind == 0) {
    __nv_bfloat16 *d = static_cast<__nv_bfloat16 *>(op) + r * 64;
#pragma unroll
    for (int c = 0; c < 64; c += 8) {
      __align__(16) __nv_bfloat16 t[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) t[u] = __float2bfloat16_rn(v[c + u]);
      *reinterpret_cast<uint4 *>(d + c) = *reinterpret_cast<const uint4 *>(t);
    }
  } else {
    float *d = static_cast<float *>(op) + r * 64;
    float *dl = op_lo + r * 64;
#pragma unroll
    for (int c = 0; c < 64; c += 4) {
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

// Writes the exact bf16 slices of one 64-wide FP64 row (K-major row r of a
// kind-3 operand with cap rows per slice plane) and its exponent.
__device__ __forceinline__ void write_slices_row(const double (&v)[64], int64_t r, int64_t cap, __nv_bfloat16 *out,
                                                 int32_t *ex) {
  uint64_t mb = 0;
#pragma unroll
  for (int c = 0; c < 64; ++c) {
    const uint64_t mc = oz_mag(v[c]);
    mb = mc > mb ? mc : mb;
  }
  const int e = oz_exponent(mb);
  ex[r] = e;
#pragma unroll
  for (int c0 = 0; c0 < 64; c0 += 8) {
    __align__(16) __nv_bfloat16 q[OZ_SLICES][8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      __nv_bfloat16 t8[OZ_SLICES];
      oz_slices(v[c0 + u], e, t8);
#pragma unroll
      for (int t = 0; t < OZ_SLICES; ++t) q[t][u] = t8[t];
    }
#pragma unroll
    for (int t = 0; t < OZ_SLICES; ++t)
      *reinterpret_cast<uint4 *>(out + ((int64_t)t * cap + r) * 64 + c0) = *reinterpret_cast<const uint4 *>(q[t]);
  }
}

// W(m x n, FP64) -= A B^T from the slices of A (rows of capA per slice) and
// B (capB), exponents eA[m], eB[n]; *err set if a bounded wait expired.
// lower: only tiles that reach the diagonal or below it (row >= boff + column
// somewhere in the tile) are updated: the trailing update of a Cholesky.
int oz_update(cudaStream_t s, int64_t m, int64_t n, const CUtensorMap &A, const CUtensorMap &B, int64_t capA,
              int64_t capB, const int32_t *eA, const int32_t *eB, double *W, int64_t ldw, int32_t *err,
              int64_t boff = 0, const int32_t *abort = nullptr, bool lower = false, bool pdl = false);

// W(m x n, column-major, ld ldw) -= A * B^T on tcgen05 (kind 0 bf16, 1 tf32,
// 2 3xTF32 with the lo maps); *err is set non-zero if a bounded wait expired.
// B's rows start at boff (a column offset into the trailing matrix).
// lower: only tiles reaching the diagonal or below it (as oz_update).
int tc_update(cudaStream_t s, int kind, int64_t m, int64_t n, const CUtensorMap &A, const CUtensorMap &B,
              const CUtensorMap &Alo, const CUtensorMap &Blo, float *W, int64_t ldw, int32_t *err, int64_t boff = 0,
              const int32_t *abort = nullptr, bool lower = false, bool pdl = false);

// The give-up test of the low-precision factorisations, from the spread
// max|u_kk| / min|u_kk| over the first `done` of `total` columns: the spread
// has reached the limit, or, once a quarter of the columns are done, its
// logarithm extrapolated linearly to the last column exceeds 100 times the
// limit (on systems with geometric spectra log(spread) grows about linearly
// with the columns factored: a kappa = 1e10 system at n = 8192 is called at
// a quarter of its columns instead of at 62%, while kappa = 1e6 systems,
// which the 3xTF32 factor refines, extrapolate below 2e4 at every step).  A
// wrong call only costs time: the factorisation that follows solves the
// system all the same.
__device__ __forceinline__ bool give_up_now(double spread, double give_up, int64_t done, int64_t total) {
  if (!(spread < give_up)) return true;
  return 4 * done >= total && spread > 1.0 && log(spread) * ((double)total / (double)done) > log(100.0 * give_up);
}

// Launch configuration of a factorisation step's kernel; pdl: a programmatic
// dependent of the previous kernel on the stream (the kernel calls
// sm100::grid_dependency_wait() before it reads what that kernel wrote), so
// the step's kernels follow each other without the launch gap.
struct StepLaunch {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[2];
  StepLaunch(dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl) {
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 0;
    if (pdl) add_pdl();
  }
  void add_pdl() {
    at[cfg.numAttrs].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[cfg.numAttrs].val.programmaticStreamSerializationAllowed = 1;
    ++cfg.numAttrs;
  }
};

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
// The LU form of a finished Cholesky factor (chol.cu): unit-lower L D^-1
// below the diagonal, D L^T on and above it (D = diag(L)); dg: n scratch.
template <typename T>
int chol_lu_form(cudaStream_t s, int64_t n, T *W, int64_t ldw, T *dg);

struct MixedLU {
  int64_t n = 0, cap_n = 0;
  int kind = -1;  // 0 bf16, 1 tf32, 2 3xTF32 update operands (FP32 W); 3 exact bf16 slices (FP64 W)
  void *aop[2] = {nullptr, nullptr}, *bop = nullptr;
  float *aop_lo[2] = {nullptr, nullptr}, *bop_lo = nullptr;
  int32_t *ea[2] = {nullptr, nullptr}, *eb = nullptr;  // kind 3: row exponents of the sliced operands
  double *sel = nullptr;  // kind 3: the current panel's pivot rows (64 x 64, row-major), from the selection
  int32_t *err = nullptr;
  int32_t *plan = nullptr;  // every panel's moves of rows (count, rows[128], src[128], per panel);
                            // then the FP64 panel's pivot rows (64)
  // running extent of |u_ii| over the panels done: [0] max, [1] min (bits of
  // non-negative doubles, ordered like the values), [2] low word = abandon flag
  uint64_t *track = nullptr;
  CUtensorMap mapA[2], mapB, mapAlo[2], mapBlo;
  CUtensorMap mapA64[2], mapAlo64[2];  // the A operands in 64-row boxes (the B side of a Cholesky update)
  cudaStream_t sp = nullptr, su = nullptr;
  cudaEvent_t ev_in = nullptr, ev_sw = nullptr, ev_wide = nullptr, ev_done = nullptr;
  int reserve(int64_t n, int kind, cudaStream_t s);
  void release(cudaStream_t s);  // frees the buffers (stream-ordered on s)
  void destroy();                // the streams and events too (device idle)
  // LU with partial pivoting of the FP32 matrix W (n x n, ld ldw) in place (kinds 0-2).
  // give_up: the factorisation is abandoned (its kernels return at once) as
  // soon as max|u_ii| / min|u_ii| over the pivots so far is not below it;
  // INFINITY never gives up.  abandoned() on the host tells afterwards.
  // perm (optional, n > 64): perm[i] = the original row in position i once
  // ipiv's interchanges are applied, kept by the swap kernels as they go.
  int factor(cudaStream_t s, float *W, int64_t ldw, int32_t *ipiv, int32_t *info, double give_up = INFINITY,
             int32_t *perm = nullptr);
  // The same for an FP64 W (kind 3).
  int factor64(cudaStream_t s, double *W, int64_t ldw, int32_t *ipiv, int32_t *info, double give_up = INFINITY,
               int32_t *perm = nullptr);
  // Cholesky W = L L^T of the lower triangle of an SPD W (chol.cu): L in the
  // lower triangle; *info = the first column whose pivot is not positive.
  int factor_chol(cudaStream_t s, float *W, int64_t ldw, int32_t *info, double give_up = INFINITY);
  int factor_chol64(cudaStream_t s, double *W, int64_t ldw, int32_t *info, double give_up = INFINITY);
};

}  // namespace bola
