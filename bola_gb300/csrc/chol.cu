// chol.cu — the low-precision Cholesky of the mixed-precision SPD solver (no
// BOLA counterpart; the FP64 answer it must reach is BOLA's potrf('L') +
// trsm solve, src/potrf.rs:101-181, src/potrf2.rs:25-80, src/trsm.rs:95-209).
//
// W = fl(D A D) (D: powers of two making the diagonal O(1)) is factored in
// place, W = L L^T, right-looking with 64-column panels, lower triangle only:
//   chol_dblock   the 64 x 64 diagonal block, in one CTA's shared memory;
//   chol_l21      L21 = W21 L11^-T, one thread per row (no pivoting, so no
//                 exchange between CTAs: the panel is a parallel solve), and
//                 the K-major operand of the update (bf16, tf32 hi/lo, or the
//                 exact bf16 slices of the FP64-accurate factor);
//   the update    W22 -= L21 L21^T on tcgen05 (tc_update / oz_update), only
//                 tiles reaching the diagonal or below it: A and B operands
//                 are the same L21 rows.
// Look-ahead as in the LU (slu.cu): the next panel's 64 columns are updated
// on the high-priority stream, the rest on the low-priority stream overlaps
// the next panel.  Afterwards chol_to_lu rewrites the factor in the LU form
// the refinement's triangular solves use: unit-lower L D^-1 below the
// diagonal, U = D L^T on and above it (D = diag(L)).
#include <cmath>

#include "common.cuh"
#include "mixed.cuh"
#include "sm100.cuh"

namespace bola {
namespace {

constexpr int CNB = 64;  // panel width = update depth

__device__ __forceinline__ float sqrtT(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrtT(double x) { return sqrt(x); }
__device__ __forceinline__ bool positive(float x) { return x > 0.f && x <= 3.4e38f; }
__device__ __forceinline__ bool positive(double x) { return x > 0.0 && x <= 1.7e308; }

__device__ __forceinline__ bool factor_stopped(const int32_t *info, const uint64_t *track) {
  return *(volatile const int32_t *)info != 0 || (track != nullptr && *(volatile const int32_t *)(track + 2) != 0);
}

// The diagonal block W[0:jb, 0:jb] (lower) = L11 L11^T, one CTA.  A pivot
// that is not positive (or not finite) stops the factorisation: *info = its
// global 1-based column, and every later kernel of the factorisation returns
// at once.  Tracks max/min of L_kk^2 (the U diagonal of the LU form) and
// gives up as the LU panel does.
template <typename T>
__global__ void __launch_bounds__(256)
chol_dblock(T *W, int64_t ldw, int jb, int32_t col0, int64_t n, int32_t *info, uint64_t *track, double give_up) {
  __shared__ T a[CNB][CNB + 1];
  __shared__ T dinv;
  __shared__ int stop;
  if (threadIdx.x == 0) stop = factor_stopped(info, track) ? 1 : 0;
  __syncthreads();
  if (stop) return;
  for (int e = threadIdx.x; e < CNB * CNB; e += blockDim.x) {
    const int i = e % CNB, j = e / CNB;
    a[i][j] = (i < jb && j < jb && i >= j) ? W[i + j * ldw] : T(0);
  }
  __syncthreads();
  double umax = 0.0, umin = INFINITY;
  int k = 0;
  for (; k < jb; ++k) {
    if (threadIdx.x == 0) {
      const T akk = a[k][k];
      if (!positive(akk)) {
        stop = 1;
        atomicCAS(info, 0, col0 + k + 1);
      } else {
        const T d = sqrtT(akk);
        a[k][k] = d;
        dinv = T(1) / d;
        umax = fmax(umax, (double)akk);
        umin = fmin(umin, (double)akk);
      }
    }
    __syncthreads();
    if (stop) break;
    const T di = dinv;
    for (int i = k + 1 + (int)threadIdx.x; i < jb; i += blockDim.x) a[i][k] *= di;
    __syncthreads();
    const int m = jb - k - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = k + 1 + e % m, j = k + 1 + e / m;
      if (i >= j) a[i][j] = fmaT(-a[i][k], a[j][k], a[i][j]);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, j = e / jb;
    if (i >= j) W[i + j * ldw] = a[i][j];
  }
  if (threadIdx.x == 0 && track != nullptr && !stop) {
    // the U diagonal of the LU form is L_kk^2 = the pivots: their running extent and the give-up test
    const uint64_t mx = (uint64_t)__double_as_longlong(umax), mn = (uint64_t)__double_as_longlong(umin);
    if (mx > track[0]) track[0] = mx;
    if (mn < track[1]) track[1] = mn;
    const double gmx = __longlong_as_double((long long)track[0]), gmn = __longlong_as_double((long long)track[1]);
    const double spread = gmn > 0.0 ? gmx / gmn : INFINITY;
    if (give_up_now(spread, give_up, col0 + jb, n)) *(volatile int32_t *)(track + 2) = 1;
  }
}

// L21 = W21 L11^-T for the rows jb..mp-1 of the panel (one thread per row,
// its 64 values in registers, L11 in shared memory), written back to W and
// as row (row - jb) of the update's K-major operand.
template <typename T, int CR>
__global__ void __launch_bounds__(CR)
chol_l21(T *W, int64_t ldw, int64_t mp, int jb, int kind, void *aop, float *aop_lo, int32_t *aexp, int64_t cap,
         const int32_t *info, const uint64_t *track) {
  __shared__ T L[CNB][CNB + 1];
  __shared__ T rd[CNB];
  __shared__ int stop;
  if (threadIdx.x == 0) stop = factor_stopped(info, track) ? 1 : 0;
  __syncthreads();
  if (stop) return;
  for (int e = threadIdx.x; e < CNB * CNB; e += CR) {
    const int i = e % CNB, j = e / CNB;
    L[i][j] = (i < jb && j < jb && i >= j) ? W[i + j * ldw] : T(0);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < CNB; k += CR) rd[k] = k < jb ? T(1) / L[k][k] : T(0);
  __syncthreads();
  const int64_t row = jb + (int64_t)blockIdx.x * CR + threadIdx.x;
  if (row >= mp) return;
  T v[CNB];
#pragma unroll
  for (int k = 0; k < CNB; ++k) v[k] = k < jb ? W[row + k * ldw] : T(0);
#pragma unroll
  for (int k = 0; k < CNB; ++k) {
    T x = v[k];
#pragma unroll
    for (int q = 0; q < k; ++q) x = fmaT(-v[q], L[k][q], x);
    v[k] = x * rd[k];  // zero beyond jb (rd = 0 there)
  }
#pragma unroll
  for (int k = 0; k < CNB; ++k)
    if (k < jb) W[row + k * ldw] = v[k];
  if (aop == nullptr) return;
  if constexpr (sizeof(T) == 4) {
    write_operand_row(kind, aop, aop_lo, row - jb, v);
  } else {
    write_slices_row(v, row - jb, cap, static_cast<__nv_bfloat16 *>(aop), aexp);
  }
}

// The diagonal of L, before chol_to_lu overwrites it.
template <typename T>
__global__ void chol_diag(int64_t n, const T *W, int64_t ldw, T *dg) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dg[i] = W[i + i * ldw];
}

// LU form of a Cholesky factor: W[i,j] = L_ij / L_jj (i > j), W[i,j] = L_ii L_ji
// (i <= j).  One CTA per 32 x 32 tile (I, J) with I >= J: it reads its lower
// tile and writes the lower tile and the transposed upper tile (J, I), which
// no other CTA touches.
template <typename T>
__global__ void __launch_bounds__(256) chol_to_lu(int64_t n, T *W, int64_t ldw, const T *dg) {
  __shared__ T t[32][33];
  const int64_t I = blockIdx.x, J = blockIdx.y;
  if (J > I) return;
  const int64_t i0 = I * 32, j0 = J * 32;
  for (int e = threadIdx.x; e < 32 * 32; e += 256) {
    const int r = e & 31, c = e >> 5;
    const int64_t i = i0 + r, j = j0 + c;
    t[r][c] = (i < n && j < n && i >= j) ? W[i + j * ldw] : T(0);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * 32; e += 256) {
    const int r = e & 31, c = e >> 5;
    const int64_t i = i0 + r, j = j0 + c;
    if (i >= n || j >= n || i < j) continue;
    if (i > j) W[i + j * ldw] = t[r][c] / dg[j];
  }
  for (int e = threadIdx.x; e < 32 * 32; e += 256) {
    const int c = e & 31, r = e >> 5;  // upper element (j0 + c, i0 + r) = L_jj L_ij, walking rows fastest
    const int64_t i = i0 + r, j = j0 + c;
    if (i >= n || j >= n || i < j) continue;
    W[j + i * ldw] = dg[j] * t[r][c];
  }
}

__global__ void zero_info(int32_t *p) { *p = 0; }
__global__ void track_reset(uint64_t *t) {
  t[0] = 0;
  t[1] = 0x7ff0000000000000ull;
  t[2] = 0;
}

template <typename T>
int chol_lookahead(MixedLU &lu, cudaStream_t s, T *W, int64_t ldw, int32_t *info, double give_up) {
  constexpr bool fp64 = sizeof(T) == 8;
  const int64_t n = lu.n;
  BOLA_TRY_CUDA(cudaEventRecord(lu.ev_in, s));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.sp, lu.ev_in, 0));
  zero_info<<<1, 1, 0, lu.sp>>>(info);
  track_reset<<<1, 1, 0, lu.sp>>>(lu.track);
  BOLA_CHECK_LAUNCH();
  BOLA_TRY_CUDA(cudaEventRecord(lu.ev_in, lu.sp));
  BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.su, lu.ev_in, 0));
  uint64_t *track = std::isinf(give_up) ? nullptr : lu.track;
  const int32_t *abort = track ? reinterpret_cast<const int32_t *>(track + 2) : nullptr;
  bool wide_pending = false;
  for (int64_t j = 0, k = 0; j < n; j += CNB, ++k) {
    const int jb = (int)imin(CNB, n - j);
    const int64_t mp = n - j;
    const bool upd = j + jb < n;
    const int buf = (int)(k & 1);
    T *Wp = W + j + j * ldw;
    {
      ProfScope prof(lu.sp, fp64 ? "chol_panel64" : "chol_panel", (double)mp * jb * jb / 2.0,
                     2.0 * sizeof(T) * (double)mp * jb, 2);
      chol_dblock<T><<<1, 256, 0, lu.sp>>>(Wp, ldw, jb, (int32_t)j, n, info, track, give_up);
      if (mp > jb) {
        constexpr int CR = fp64 ? 64 : 128;
        chol_l21<T, CR><<<(unsigned)cdiv(mp - jb, CR), CR, 0, lu.sp>>>(
            Wp, ldw, mp, jb, lu.kind, upd ? lu.aop[buf] : nullptr, fp64 ? nullptr : lu.aop_lo[buf],
            fp64 ? lu.ea[buf] : nullptr, lu.cap_n, info, track);
      }
      BOLA_CHECK_LAUNCH();
    }
    if (!upd) continue;
    // the update of step k writes columns the previous wide update also writes
    if (wide_pending) BOLA_TRY_CUDA(cudaStreamWaitEvent(lu.sp, lu.ev_wide, 0));
    wide_pending = false;
    const int64_t m2 = mp - jb, n2 = n - j - jb;
    const int64_t nb_next = imin(CNB, n2);
    T *W22 = W + (j + jb) + (j + jb) * ldw;
    auto update = [&](cudaStream_t st, int64_t cols, int64_t boff) -> int {
      if constexpr (fp64)
        return oz_update(st, m2, cols, lu.mapA[buf], lu.mapA64[buf], lu.cap_n, lu.cap_n, lu.ea[buf], lu.ea[buf],
                         W22 + boff * ldw, ldw, lu.err, boff, abort, true);
      else
        return tc_update(st, lu.kind, m2, cols, lu.mapA[buf], lu.mapA64[buf], lu.mapAlo[buf], lu.mapAlo64[buf],
                         W22 + boff * ldw, ldw, lu.err, boff, abort, true);
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

}  // namespace

int MixedLU::factor_chol(cudaStream_t s, float *W, int64_t ldw, int32_t *info, double give_up) {
  return chol_lookahead<float>(*this, s, W, ldw, info, give_up);
}

int MixedLU::factor_chol64(cudaStream_t s, double *W, int64_t ldw, int32_t *info, double give_up) {
  return chol_lookahead<double>(*this, s, W, ldw, info, give_up);
}

// The LU form of a finished Cholesky factor (see chol_to_lu); dg: n scratch elements.
template <typename T>
int chol_lu_form(cudaStream_t s, int64_t n, T *W, int64_t ldw, T *dg) {
  ProfScope prof(s, "chol_to_lu", 0.0, 3.0 * sizeof(T) * (double)n * n / 2.0, 2);
  chol_diag<T><<<(unsigned)cdiv(n, 256), 256, 0, s>>>(n, W, ldw, dg);
  const unsigned nt = (unsigned)cdiv(n, 32);
  chol_to_lu<T><<<dim3(nt, nt), 256, 0, s>>>(n, W, ldw, dg);
  BOLA_CHECK_LAUNCH();
  return 0;
}
template int chol_lu_form<float>(cudaStream_t, int64_t, float *, int64_t, float *);
template int chol_lu_form<double>(cudaStream_t, int64_t, double *, int64_t, double *);

}  // namespace bola

// The low-precision Cholesky alone, for tests and profiling: the lower
// triangle of W (n x n FP32, SPD) is replaced by L (W = L L^T); *info
// (device) = the first column whose pivot is not positive, or 0.  Synchronous.
extern "C" int bola_spotrf_mixed(int kind, int64_t n, float *w, int64_t ldw, int32_t *info, bola_stream_t stream) {
  using namespace bola;
  if (kind < 0 || kind > 2) return -1;
  if (n < 0 || n > 8192) return -2;
  if (ldw < imax(1, n)) return -4;
  if (n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  MixedLU lu;
  int st = lu.reserve(n, kind, s);
  if (st == 0) st = lu.factor_chol(s, w, ldw, info);
  int32_t err = 0;
  if (st == 0 && lu.err) st = cudaMemcpyAsync(&err, lu.err, sizeof err, cudaMemcpyDeviceToHost, s) == cudaSuccess ? 0 : BOLA_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess && st == 0) st = cuda_fail(cudaGetLastError(), "bola_spotrf_mixed");
  lu.destroy();
  if (st == 0 && err != 0) st = fail(BOLA_ERR_CUDA, "mixed Cholesky: a bounded wait expired (code %d)", err);
  return st;
}
