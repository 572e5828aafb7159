// level1.cu — idamax, scal, ger, dot, axpy and laswp with BOLA's rounding.
//
// These are HBM/latency-bound helpers (BOLA's src/idamax.rs, src/scal.rs,
// src/ger.rs, src/utilities.rs, src/laswp.rs).  Inside getrf they are fused
// into the panel and swap kernels; the entry points here are the standalone
// drop-ins.
#include "common.cuh"

namespace bola {
namespace {

// ---- idamax: two-pass argmax under BOLA's lane order ----------------------
__global__ void idamax_pass1(int64_t n, const double *__restrict__ x, int lanes, Cand *out) {
  __shared__ Cand sh[32];
  Cand best = cand_none();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Cand c = make_cand(x[i], i, n, lanes);
    if (cand_better(c, best)) best = c;
  }
  best = warp_best(best);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = best;
  __syncthreads();
  if (w == 0) {
    best = (l < (int)(blockDim.x >> 5)) ? sh[l] : cand_none();
    best = warp_best(best);
    if (l == 0) out[blockIdx.x] = best;
  }
}

__global__ void idamax_pass2(int64_t nc, const Cand *__restrict__ in, int64_t *result) {
  __shared__ Cand sh[32];
  Cand best = cand_none();
  for (int64_t i = threadIdx.x; i < nc; i += blockDim.x)
    if (cand_better(in[i], best)) best = in[i];
  best = warp_best(best);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = best;
  __syncthreads();
  if (w == 0) {
    best = (l < (int)(blockDim.x >> 5)) ? sh[l] : cand_none();
    best = warp_best(best);
    // BOLA returns index 0 when nothing beats its starting maximum.
    if (l == 0) *result = best.v < 0 ? 0 : best.idx;
  }
}

__global__ void write_i64(int64_t *p, int64_t v) { *p = v; }

// ---- scal (src/scal.rs:45-57) ----------------------------------------------
__global__ void scal_kernel(int64_t n, double alpha, double *x, int64_t incx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i * incx] = __dmul_rn(x[i * incx], alpha);
}
__global__ void scal_zero_stride(int64_t n, double alpha, double *x) {
  double v = x[0];
  for (int64_t i = 0; i < n; ++i) v = __dmul_rn(v, alpha);
  x[0] = v;
}

// ---- ger (src/ger.rs:28-61) -----------------------------------------------
__global__ void ger_kernel(int64_t m, int64_t n, double alpha, const double *__restrict__ x,
                           const double *__restrict__ y, int64_t ldy, double *__restrict__ a,
                           int64_t lda, int lanes) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * n) return;
  const int64_t i = e % m, j = e / m;
  const int64_t n_unrolled = n - (n % 2);
  const int64_t rows_vec = (m / lanes) * lanes;
  double *ap = a + i + j * lda;
  if (j < n_unrolled) {
    const int64_t j0 = j & ~(int64_t)1;
    const double t0 = __dmul_rn(alpha, y[j0 * ldy]);
    const double t1 = __dmul_rn(alpha, y[(j0 + 1) * ldy]);
    if (!nonzero64(t0) && !nonzero64(t1)) return;
    const double t = (j == j0) ? t0 : t1;
    *ap = fused_or_unfused(i < rows_vec, x[i], t, *ap);
  } else {
    const double t = __dmul_rn(alpha, y[j * ldy]);
    if (nonzero64(t)) *ap = add_prod(*ap, t, x[i]);
  }
}

// ---- dot (src/utilities.rs:22-92) -------------------------------------------
__global__ void dot_kernel(int64_t n, const double *x, int64_t incx, const double *y, int64_t incy,
                           int lanes, double *result) {
  double s;
  if (incx == 1 && incy == 1) {
    s = dot_exact(n, x, 1, y, 1, lanes);
  } else {
    s = 0.0;
    for (int64_t i = 0; i < n; ++i) s = add_prod(s, x[i * incx], y[i * incy]);
  }
  *result = s;
}

// ---- axpy (src/utilities.rs:107-164) ----------------------------------------
__global__ void axpy_kernel(int64_t n, double alpha, const double *x, int64_t incx, double *y,
                            int64_t incy, int lanes) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (incx == 1 && incy == 1) {
    y[i] = daxpy_elem(y[i], alpha, x[i], i, n, lanes);
  } else {
    y[i * incy] = add_prod(y[i * incy], alpha, x[i * incx]);
  }
}
__global__ void axpy_zero_stride(int64_t n, double alpha, const double *x, int64_t incx, double *y) {
  double v = y[0];
  for (int64_t i = 0; i < n; ++i) v = add_prod(v, alpha, x[i * incx]);
  y[0] = v;
}

// ---- laswp (src/laswp.rs:22-132) --------------------------------------------
// Every column receives the same ordered list of row interchanges.  Short
// lists (at most 32 interchanges, the getrf panel case) are composed once per
// block into "row r takes the old value of row src(r)" and applied by a warp
// per column; long lists are walked in order by one thread per column.
__global__ void laswp_short(int64_t n, double *A, int64_t lda, SwapPlan plan, const int32_t *ipiv,
                            const int32_t *info) {
  __shared__ int64_t rows[64], src[64];
  __shared__ int cnt;
  if (stop_flag(info)) return;
  if (threadIdx.x < 32) {
    const int c = compose_swaps_warp(plan, ipiv, rows, src);
    if (threadIdx.x == 0) cnt = c;
  }
  __syncthreads();
  const int warps = blockDim.x >> 5, lane = threadIdx.x & 31;
  const int64_t col = (int64_t)blockIdx.x * warps + (threadIdx.x >> 5);
  if (col >= n) return;
  double *cp = A + col * lda;
  const double v0 = lane < cnt ? cp[src[lane]] : 0.0;
  const double v1 = lane + 32 < cnt ? cp[src[lane + 32]] : 0.0;
  __syncwarp();
  if (lane < cnt) cp[rows[lane]] = v0;
  if (lane + 32 < cnt) cp[rows[lane + 32]] = v1;
}

__global__ void laswp_long(int64_t n, double *A, int64_t lda, SwapPlan p, const int32_t *ipiv,
                           const int32_t *info) {
  if (stop_flag(info)) return;
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= n) return;
  double *cp = A + col * lda;
  int64_t ix = p.ix0;
  for (int32_t i = p.i1; p.i_inc > 0 ? i <= p.i2 : i >= p.i2; i += p.i_inc, ix += p.incx) {
    const int64_t ip = ipiv[ix];
    if (ip != (int64_t)i) {
      const double t = cp[i - 1];
      cp[i - 1] = cp[ip - 1];
      cp[ip - 1] = t;
    }
  }
}

__global__ void ipiv_add_kernel(int32_t *ipiv, int64_t count, int32_t add, const int32_t *info) {
  if (stop_flag(info)) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) ipiv[i] += add;
}

}  // namespace

int laswp_exact(cudaStream_t s, int64_t n, double *A, int64_t lda, int32_t k1, int32_t k2,
                const int32_t *ipiv, int32_t incx, const int32_t *info) {
  if (n <= 0 || incx == 0 || k1 > k2) return 0;
  SwapPlan p;
  if (incx > 0) {
    p.ix0 = k1 - 1;
    p.i1 = k1;
    p.i2 = k2;
    p.i_inc = 1;
  } else {
    p.ix0 = (int64_t)(k1 - 1) + (int64_t)(k2 - k1) * (-(int64_t)incx);
    p.i1 = k2;
    p.i2 = k1;
    p.i_inc = -1;
  }
  p.incx = incx;
  ProfScope prof(s, "laswp", 0.0, 32.0 * (double)n * ((int64_t)k2 - k1 + 1));
  if ((int64_t)k2 - k1 + 1 <= 32) {
    const int warps = 8;
    laswp_short<<<(unsigned)cdiv(n, warps), 32 * warps, 0, s>>>(n, A, lda, p, ipiv, info);
  } else {
    laswp_long<<<(unsigned)cdiv(n, 128), 128, 0, s>>>(n, A, lda, p, ipiv, info);
  }
  BOLA_CHECK_LAUNCH();
  return 0;
}

int ipiv_add(cudaStream_t s, int32_t *ipiv, int64_t count, int32_t add, const int32_t *info) {
  if (count <= 0 || add == 0) return 0;
  ProfScope prof(s, "ipiv_add");
  ipiv_add_kernel<<<(unsigned)cdiv(count, 256), 256, 0, s>>>(ipiv, count, add, info);
  BOLA_CHECK_LAUNCH();
  return 0;
}

}  // namespace bola

using namespace bola;

extern "C" {

int bola_idamax(int64_t n, const double *x, int64_t *result, bola_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (n < 0) return -1;
  if (n == 0) {
    write_i64<<<1, 1, 0, s>>>(result, 0);
    BOLA_CHECK_LAUNCH();
    return 0;
  }
  const int64_t nb = imin(cdiv(n, 2048), 2 * (int64_t)num_sms());
  Scratch tmp;
  BOLA_TRY(tmp.alloc(sizeof(Cand) * nb, s));
  idamax_pass1<<<(unsigned)nb, 256, 0, s>>>(n, x, lanes(), tmp.as<Cand>());
  BOLA_CHECK_LAUNCH();
  idamax_pass2<<<1, 1024, 0, s>>>(nb, tmp.as<Cand>(), result);
  BOLA_CHECK_LAUNCH();
  return 0;
}

int bola_dscal(int64_t n, double alpha, double *x, int64_t incx, bola_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (n < 0) return -1;
  if (incx < 0) return -4;
  if (n == 0) return 0;
  if (incx == 0) {
    scal_zero_stride<<<1, 1, 0, s>>>(n, alpha, x);
  } else {
    scal_kernel<<<(unsigned)cdiv(n, 256), 256, 0, s>>>(n, alpha, x, incx);
  }
  BOLA_CHECK_LAUNCH();
  return 0;
}

int bola_dger(int64_t m, int64_t n, double alpha, const double *x, const double *y, int64_t ldy,
              double *a, int64_t lda, bola_stream_t stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (m == 0 || n == 0) return 0;
  if (ldy < 0) return -6;
  if (lda < imax(1, m)) return -8;
  ger_kernel<<<(unsigned)cdiv(m * n, 256), 256, 0, (cudaStream_t)stream>>>(m, n, alpha, x, y, ldy, a, lda,
                                                                           lanes());
  BOLA_CHECK_LAUNCH();
  return 0;
}

int bola_ddot(int64_t n, const double *x, int64_t incx, const double *y, int64_t incy, double *result,
              bola_stream_t stream) {
  if (n < 0) return -1;
  if (incx < 0) return -3;
  if (incy < 0) return -5;
  dot_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(n, x, incx, y, incy, lanes(), result);
  BOLA_CHECK_LAUNCH();
  return 0;
}

int bola_daxpy(int64_t n, double alpha, const double *x, int64_t incx, double *y, int64_t incy,
               bola_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (n < 0) return -1;
  if (incx < 0) return -4;
  if (incy < 0) return -6;
  if (n == 0 || alpha == 0.0) return 0;
  if (incy == 0) {
    axpy_zero_stride<<<1, 1, 0, s>>>(n, alpha, x, incx, y);
  } else {
    axpy_kernel<<<(unsigned)cdiv(n, 256), 256, 0, s>>>(n, alpha, x, incx, y, incy, lanes());
  }
  BOLA_CHECK_LAUNCH();
  return 0;
}

int bola_dlaswp(int64_t n, double *a, int64_t lda, int32_t k1, int32_t k2, const int32_t *ipiv,
                int32_t incx, bola_stream_t stream) {
  if (n < 0) return -1;
  if (n == 0 || incx == 0 || k1 > k2) return 0;
  if (k1 < 1) return -4;
  if (lda < 1) return -3;
  return laswp_exact((cudaStream_t)stream, n, a, lda, k1, k2, ipiv, incx, nullptr);
}

}  // extern "C"
