// oz_residual.cu — FP64-accurate matrix products A X (n x n times n x nrhs)
// on the bf16 tensor cores, for the residuals r = b - A x and the GMRES
// products of the mixed-precision refinement (no BOLA counterpart).
//
// GB300 retires about two FP64 fused multiply-adds per clock per SM, so an
// FP64 product with 16 right-hand sides at n = 8192 (4.3 GFLOP) takes ~2 ms
// on the FP64 pipe.  Here A is split once per solve, exactly, into
// OZ_SA = 7 planes of signed 8-bit digits under a power-of-two scale per row
// (the Ozaki scheme):
//     a_ij = 2^(e_i - 7) sum_t s_ijt 2^(-8t)     (to within 2^(e_i - 56)),
// and each right-hand side column into OZ_SX = 8 such planes under a scale
// per column.  Digits are integers with |s| <= 128, exact in bf16, so a digit
// product is an integer below 2^14 and a sum of 512 of them stays at or
// below 2^23: the tensor core's FP32 accumulator holds every such partial sum
// exactly, whatever its order.  For every pair of planes (t, u) with
// t + u <= OZ_D = 7 (36 pairs), each 512-deep K chunk is accumulated in TMEM,
// converted to an integer and added, shifted by its weight, into two 64-bit
// fixed-point sums per output (weights 0..3 and 4..7).  Those integer sums
// are exact, and K-split partial sums combine exactly with 64-bit atomics.
// The dropped pairs and the digit rounding bound the error per output by
// about 2^-46 * n * max_j|a_ij| * max|x_c|, the order of an FP64 dot
// product's own rounding bound; in practice the result is the exact product
// rounded once or twice.
//
// Per CTA: a 128-row tile of A and a range of K chunks.  Warp 0 streams A's
// digit tiles (128 x 64, 16 KB) and the x digits (16 rows per plane) through
// a four-stage TMA ring; warp 1 issues the tcgen05.mma chains (M = 128,
// N = 16 (8 - t), K = 16) into one of two 128-column TMEM accumulators;
// warps 2-5 drain the other accumulator into their fixed-point registers.
// A's digit planes are read once per product: the kernel is HBM-bound at
// 7 x 2 bytes per element of A.
#include <cuda_bf16.h>

#include <cstring>

#include "common.cuh"
#include "mixed.cuh"
#include "sm100.cuh"

namespace bola {
namespace {

using namespace sm100;

constexpr int SA = OZ_SA, SX = OZ_SX, DMAX = OZ_D;
constexpr int RM = 128;           // rows per tile
constexpr int KS = 64;            // K per stage (one 128-byte swizzled row)
constexpr int KCH = 512;          // K per exact accumulation chunk
constexpr int NRB = 16;           // right-hand sides per product
constexpr int NST = 4;            // pipeline stages
constexpr int A_TILE = RM * 128;  // 16 KB
constexpr int X_TILE = 128 * 128; // up to 8 planes x 16 rows
constexpr int STAGE = A_TILE + X_TILE;
constexpr int OZR_SMEM = NST * STAGE + 1024;
constexpr int OZR_THREADS = 192;
constexpr int32_t NONFINITE = 0x7fffffff;  // exponent marker of a row or column holding Inf or NaN

// The digits of v (|v| < 2^e) in NS planes, with integer operations only:
// X = round(v 2^(8 NS - 1 - e)), then signed base-256 digits, most
// significant first: v ~ 2^(e - 7) sum_t s_t 2^(-8t), |s_t| <= 128.
template <int NS>
__device__ __forceinline__ void digits(double v, int e, int32_t (&s)[NS]) {
  const uint64_t bits = (uint64_t)__double_as_longlong(v);
  const int ev = (int)((bits >> 52) & 0x7FF);
  int64_t X = 0;
  if (ev != 0) {
    const uint64_t M = (bits & ((1ull << 52) - 1)) | (1ull << 52);  // v = M 2^(ev - 1075)
    const int k = 1076 - 8 * NS - ev + e;                            // X = M 2^-k
    if (k <= 0) X = (int64_t)(M << (-k));                           // (k >= 1012 - 1022 for NS <= 8)
    else if (k < 64) X = (int64_t)((M + (1ull << (k - 1))) >> k);
    if (bits >> 63) X = -X;
  }
#pragma unroll
  for (int t = NS - 1; t > 0; --t) {
    const int d = (int)((X + 128) & 255) - 128;
    s[t] = d;
    X = (X - d) >> 8;
  }
  s[0] = (int32_t)X;
}

// e with max|v| in [2^(e-1), 2^e) from the largest |v|'s bits; NONFINITE for Inf/NaN
__device__ __forceinline__ int32_t exponent_of(uint64_t mag_bits) {
  if (mag_bits >= 0x7ff0000000000000ull) return NONFINITE;
  return oz_exponent(mag_bits);
}

// Row statistics of A in one pass: max|a_ij| (as ordered bits, atomicMax)
// and, per 512-column block, the partial row sums of |a_ij| (summed in a
// fixed order afterwards: the norm must not depend on scheduling).  CTA:
// 128 rows x 512 columns, two column halves of 256 threads.
__global__ void __launch_bounds__(256)
oz_row_stats(int64_t n, const double *__restrict__ A, int64_t lda, unsigned long long *rmax, double *psum) {
  __shared__ double red[128];
  __shared__ unsigned long long mred[128];
  const int r = threadIdx.x & 127, h = threadIdx.x >> 7;
  const int64_t i = (int64_t)blockIdx.x * 128 + r;
  const int64_t c0 = (int64_t)blockIdx.y * KCH;
  const int64_t c1 = imin(n, c0 + KCH);
  double s = 0.0;
  uint64_t m = 0;
  if (i < n)
    for (int64_t c = c0 + h; c < c1; c += 2) {
      const double v = A[i + c * lda];
      s += fabs(v);
      const uint64_t b = oz_mag(v);
      m = b > m ? b : m;
    }
  if (h == 1) {
    red[r] = s;
    mred[r] = m;
  }
  __syncthreads();
  if (h == 0 && i < n) {
    s += red[r];
    m = mred[r] > m ? mred[r] : m;
    psum[(int64_t)blockIdx.y * n + i] = s;
    atomicMax(rmax + i, (unsigned long long)m);
  }
}

// rowsum[i] = sum of the partial sums in block order; e[i] from the row max.
__global__ void oz_row_finish(int64_t n, int nblk, const unsigned long long *rmax, const double *psum, double *rowsum,
                              int32_t *e) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += psum[(int64_t)b * n + i];
  if (rowsum) rowsum[i] = s;
  e[i] = exponent_of(rmax[i]);
}

// A's digit planes, row-major: plane t, row i at ((t * mrows + i) * kp).
// CTA: a 64 x 64 tile, staged through shared memory (column-major in, rows out).
__global__ void __launch_bounds__(256)
oz_split_matrix(int64_t n, const double *__restrict__ A, int64_t lda, const int32_t *__restrict__ e, int64_t mrows,
                int64_t kp, __nv_bfloat16 *__restrict__ out) {
  __shared__ double T[64][65];
  const int64_t i0 = (int64_t)blockIdx.y * 64, j0 = (int64_t)blockIdx.x * 64;
  for (int q = threadIdx.x; q < 64 * 64; q += 256) {
    const int r = q & 63, c = q >> 6;
    T[r][c] = (i0 + r < n && j0 + c < n) ? A[(i0 + r) + (j0 + c) * lda] : 0.0;
  }
  __syncthreads();
  // thread: row r, columns 2p and 2p + 1 (a warp writes 128 contiguous bytes per plane)
  for (int q = threadIdx.x; q < 64 * 32; q += 256) {
    const int p = q & 31, r = q >> 5;
    const int64_t i = i0 + r, j = j0 + 2 * p;
    if (i >= n || j >= n) continue;
    const int32_t ei = e[i];
    int32_t d0[SA], d1[SA];
    if (ei == NONFINITE) {
#pragma unroll
      for (int t = 0; t < SA; ++t) d0[t] = d1[t] = 0;
    } else {
      digits<SA>(T[r][2 * p], ei, d0);
      digits<SA>(T[r][2 * p + 1], ei, d1);
    }
#pragma unroll
    for (int t = 0; t < SA; ++t) {
      __nv_bfloat162 w;
      w.x = __int2bfloat16_rn(d0[t]);
      w.y = __int2bfloat16_rn(d1[t]);
      *reinterpret_cast<__nv_bfloat162 *>(out + ((int64_t)t * mrows + i) * kp + j) = w;
    }
  }
}

// The right-hand sides' digit planes: plane u, column c (< 16) at row
// (u * 16 + c) of a row-major array (pitch kp); columns c >= nr are zero.
// One CTA per column: its max, then its digits.
__global__ void __launch_bounds__(1024)
oz_split_rhs(int64_t n, int nr, const double *__restrict__ x, int64_t ldx, int64_t kp, __nv_bfloat16 *__restrict__ out,
             int32_t *f) {
  __shared__ unsigned long long red[32];
  __shared__ int32_t fe;
  const int c = blockIdx.x;
  const double *xc = x + (int64_t)c * ldx;
  uint64_t m = 0;
  if (c < nr)
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const uint64_t b = oz_mag(xc[i]);
      m = b > m ? b : m;
    }
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t o = __shfl_xor_sync(0xffffffffu, m, off);
    m = o > m ? o : m;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t mm = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mm = red[w] > mm ? red[w] : mm;
    fe = exponent_of(mm);
    f[c] = fe;
  }
  __syncthreads();
  const int32_t ec = fe;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    int32_t d[SX];
    if (c < nr && ec != NONFINITE) {
      digits<SX>(xc[i], ec, d);
    } else {
#pragma unroll
      for (int u = 0; u < SX; ++u) d[u] = 0;
    }
#pragma unroll
    for (int u = 0; u < SX; ++u) out[((int64_t)u * NRB + c) * kp + i] = __int2bfloat16_rn(d[u]);
  }
}

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


// acc (int64, [2][n][16]): += the fixed-point sums of this CTA's rows over its K chunks.
__global__ void __launch_bounds__(OZR_THREADS, 1)
oz_product_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapX, int64_t n,
                  int64_t mrows, int chunks_per_cta, unsigned long long *acc, int32_t *err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[NST], empty[NST], tfull[2], tempty[2];
  __shared__ uint32_t tmem_slot;
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t m0 = (int64_t)blockIdx.x * RM;
  const int nchunks = (int)cdiv(n, KCH);
  const int ch0 = blockIdx.y * chunks_per_cta;
  const int ch1 = (int)imin(nchunks, ch0 + chunks_per_cta);
  const int nch = ch1 > ch0 ? ch1 - ch0 : 0;
  const int units = SA * nch;  // (plane t, chunk) pairs, t outer

  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 4);
    }
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(&tmem_slot, 256);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // -- producer: A's digit tile and the x digits of the planes paired with it
    if (lane == 0) {
      int it = 0;
      for (int un = 0; un < units && *(volatile int32_t *)err == 0; ++un) {
        const int t = un / nch, ch = ch0 + un % nch;
        const int nx = NRB * (DMAX - t + 1) / 16;  // 16-row x boxes
        const int64_t k0 = (int64_t)ch * KCH;
        const int ks = (int)imin(KCH / KS, cdiv(n - k0, KS));
        for (int q = 0; q < ks; ++q, ++it) {
          const int s = it % NST;
          if (!bounded_wait(&empty[s], ((it / NST) & 1) ^ 1)) {
            atomicExch(err, 11);
            break;
          }
          uint8_t *st = base + s * STAGE;
          mbar_arrive_expect_tx(&full[s], A_TILE + nx * 2048);
          const int32_t kx = (int32_t)(k0 + q * KS);
          tma_load_2d(st, &mapA, kx, (int32_t)(t * mrows + m0), &full[s]);
          for (int b = 0; b < nx; ++b) tma_load_2d(st + A_TILE + b * 2048, &mapX, kx, b * 16, &full[s]);
        }
      }
    }
  } else if (warp == 1) {
    // -- MMA issuer: one accumulator per (plane, chunk), alternating TMEM halves
    if (lane == 0) {
      int it = 0;
      for (int un = 0; un < units; ++un) {
        const int t = un / nch, ch = ch0 + un % nch;
        const int N = NRB * (DMAX - t + 1);
        const uint32_t idesc = make_idesc(1u, RM, N);
        const int b = un & 1;
        const int64_t k0 = (int64_t)ch * KCH;
        const int ks = (int)imin(KCH / KS, cdiv(n - k0, KS));
        if (!bounded_wait(&tempty[b], ((un >> 1) & 1) ^ 1)) {
          atomicExch(err, 12);
          break;
        }
        tc_fence_after();
        bool ok = true;
        for (int q = 0; q < ks; ++q, ++it) {
          const int s = it % NST;
          if (!bounded_wait(&full[s], (it / NST) & 1)) {
            atomicExch(err, 13);
            ok = false;
            break;
          }
          tc_fence_after();
          uint8_t *st = base + s * STAGE;
          const uint64_t da = sw128_kmajor_desc(st), db = sw128_kmajor_desc(st + A_TILE);
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma<0>(tmem + (uint32_t)(b * 128), desc_advance(da, kk * 32), desc_advance(db, kk * 32), idesc,
                    (q > 0 || kk > 0) ? 1u : 0u);
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&tfull[b]);
      }
    }
  } else {
    // -- epilogue: warps 2-5 own TMEM lanes 32 (warp % 4) ..: one row each
    const int qd = warp & 3;
    const int64_t row = m0 + qd * 32 + lane;
    long long hi[NRB], lo[NRB];
#pragma unroll
    for (int c = 0; c < NRB; ++c) hi[c] = lo[c] = 0;
    bool ok = true;
    for (int un = 0; un < units; ++un) {
      const int t = un / nch;
      const int b = un & 1;
      if (!bounded_wait(&tfull[b], (un >> 1) & 1)) {
        atomicExch(err, 14);
        ok = false;
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int u = 0; u <= DMAX; ++u) {
        if (u > DMAX - t) break;
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(b * 128 + u * 16), v);
        const int d = t + u;  // weight 2^(-8d)
#pragma unroll
        for (int c = 0; c < NRB; ++c) {
          const long long iv = (long long)__float2int_rn(v[c]);  // exact: |v| <= 2^23
          if (d <= 3) hi[c] += iv << (8 * (3 - d));
          else lo[c] += iv << (8 * (7 - d));
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);
    }
    if (ok && row < n) {
#pragma unroll
      for (int c = 0; c < NRB; ++c) {
        atomicAdd(acc + row * NRB + c, (unsigned long long)hi[c]);
        atomicAdd(acc + ((int64_t)n + row) * NRB + c, (unsigned long long)lo[c]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, 256);
}

// v * 2^k for an exact power of two built from bits (|k| within the normal range)
__device__ __forceinline__ double scale2(double v, int k) {
  if (k < -1022 || k > 1023) return ldexp(v, k);
  return v * __longlong_as_double((long long)((uint64_t)(k + 1023) << 52));
}

// out = b - A x (b given) or A x, from the fixed-point sums; columns c < nr.
__global__ void oz_product_finish(int64_t n, int nr, int c0, const unsigned long long *acc, const int32_t *e,
                                  const int32_t *f, const double *b, int64_t ldb, double *out, int64_t ldo) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n * nr) return;
  const int64_t i = q % n;
  const int c = (int)(q / n);
  const int32_t ei = e[i], fc = f[c];
  double val;
  if (ei == NONFINITE || fc == NONFINITE) {
    val = __longlong_as_double(0x7ff8000000000000ll);  // NaN: a non-finite operand
  } else {
    const long long hi = (long long)acc[i * NRB + c], lo = (long long)acc[(n + i) * NRB + c];
    const int E = ei + fc - 14;
    val = scale2((double)hi, E - 24) + scale2((double)lo, E - 56);
  }
  double *o = out + i + (int64_t)(c0 + c) * ldo;
  *o = b != nullptr ? b[i + (int64_t)(c0 + c) * ldb] - val : val;
}

}  // namespace

int OzMatrix::reserve(int64_t n_) {
  if (n_ <= cap) {
    n = n_;
    return 0;
  }
  release();
  const int64_t mr = cdiv(n_, RM) * RM, k = cdiv(n_, KS) * KS;
  auto al = [](void **p, size_t b) -> int {
    return cudaMalloc(p, b) == cudaSuccess ? 0 : fail(BOLA_ERR_CUDA, "oz product: out of memory (%zu bytes)", b);
  };
  BOLA_TRY(al(reinterpret_cast<void **>(&planes), sizeof(__nv_bfloat16) * SA * mr * k));
  BOLA_TRY(al(reinterpret_cast<void **>(&xplanes), sizeof(__nv_bfloat16) * SX * NRB * k));
  BOLA_TRY(al(reinterpret_cast<void **>(&e), sizeof(int32_t) * mr));
  BOLA_TRY(al(reinterpret_cast<void **>(&f), sizeof(int32_t) * NRB));
  BOLA_TRY(al(reinterpret_cast<void **>(&rmax), sizeof(unsigned long long) * mr));
  BOLA_TRY(al(reinterpret_cast<void **>(&psum), sizeof(double) * cdiv(n_, KCH) * n_));
  BOLA_TRY(al(reinterpret_cast<void **>(&acc), sizeof(unsigned long long) * 2 * NRB * mr));
  bytes = (int64_t)(sizeof(__nv_bfloat16) * (SA * mr * k + SX * NRB * k) + sizeof(int32_t) * (mr + NRB) +
                    sizeof(unsigned long long) * 3 * mr + sizeof(double) * cdiv(n_, KCH) * n_);
  cap = n_;
  n = n_;
  mrows = mr;
  kp = k;
  return 0;
}

void OzMatrix::release() {
  for (void *p : {(void *)planes, (void *)xplanes, (void *)e, (void *)f, (void *)rmax, (void *)psum, (void *)acc})
    if (p) cudaFree(p);
  planes = xplanes = nullptr;
  e = f = nullptr;
  rmax = acc = nullptr;
  psum = nullptr;
  cap = n = mrows = kp = bytes = 0;
  ready = false;
}

// Splits A into its digit planes (and ||A||_inf's row sums into rowsum, if given).
int OzMatrix::split(cudaStream_t s, const double *A, int64_t lda, double *rowsum) {
  ProfScope prof(s, "oz_split", 0.0, 8.0 * 2.0 * n * n + 2.0 * SA * n * n, 4);
  const int nblk = (int)cdiv(n, KCH);
  BOLA_TRY_CUDA(cudaMemsetAsync(rmax, 0, sizeof(unsigned long long) * n, s));
  oz_row_stats<<<dim3((unsigned)cdiv(n, 128), (unsigned)nblk), 256, 0, s>>>(n, A, lda, rmax, psum);
  oz_row_finish<<<(unsigned)cdiv(n, 256), 256, 0, s>>>(n, nblk, rmax, psum, rowsum, e);
  oz_split_matrix<<<dim3((unsigned)cdiv(n, 64), (unsigned)cdiv(n, 64)), 256, 0, s>>>(n, A, lda, e, mrows, kp, planes);
  BOLA_CHECK_LAUNCH();
  BOLA_TRY(make_kmajor_map2(&mapA, planes, n, SA * mrows, kp, RM));
  BOLA_TRY(make_kmajor_map2(&mapX, xplanes, n, SX * NRB, kp, 16));
  ready = true;
  return 0;
}

// out = b - A x (b != nullptr) or out = A x, for nr right-hand sides (any
// count: blocks of 16).  *err is set if a bounded wait inside expired.
int OzMatrix::product(cudaStream_t s, int nr, const double *x, int64_t ldx, const double *b, int64_t ldb, double *out,
                      int64_t ldo, int32_t *err) {
  if (!ready) return fail(BOLA_ERR_CUDA, "oz product: matrix not split");
  static bool attr = false;
  if (!attr) {
    BOLA_TRY_CUDA(cudaFuncSetAttribute(oz_product_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZR_SMEM));
    attr = true;
  }
  const int mt = (int)cdiv(n, RM);
  const int nchunks = (int)cdiv(n, KCH);
  const int split = (int)imax(1, imin(nchunks, num_sms() / mt));
  const int cpc = (int)cdiv(nchunks, split);
  const int grid_y = (int)cdiv(nchunks, cpc);
  for (int c0 = 0; c0 < nr; c0 += NRB) {
    const int nb = (int)imin(NRB, nr - c0);
    ProfScope prof(s, "oz_product", 2.0 * (double)n * n * nb, 2.0 * SA * (double)n * n, 4);
    BOLA_TRY_CUDA(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * 2 * NRB * n, s));
    oz_split_rhs<<<NRB, 1024, 0, s>>>(n, nb, x + (int64_t)c0 * ldx, ldx, kp, xplanes, f);
    oz_product_kernel<<<dim3((unsigned)mt, (unsigned)grid_y), OZR_THREADS, OZR_SMEM, s>>>(mapA, mapX, n, mrows, cpc,
                                                                                          acc, err);
    oz_product_finish<<<(unsigned)cdiv(n * nb, 256), 256, 0, s>>>(n, nb, c0, acc, e, f, b, ldb, out, ldo);
    BOLA_CHECK_LAUNCH();
  }
  return 0;
}

}  // namespace bola

// FP64-accurate product on the tensor cores, for tests and profiling:
// out = b - A x (b != NULL) or A x.  Allocates its digit planes per call.
extern "C" int bola_dgemv_oz(int64_t n, int64_t nrhs, const double *a, int64_t lda, const double *x, int64_t ldx,
                             const double *b, int64_t ldb, double *out, int64_t ldo, bola_stream_t stream) {
  using namespace bola;
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (lda < imax(1, n)) return -4;
  if (ldx < imax(1, n)) return -6;
  if (b != nullptr && ldb < imax(1, n)) return -8;
  if (ldo < imax(1, n)) return -10;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  OzMatrix M;
  int32_t *err = nullptr;
  int st = M.reserve(n);
  if (st == 0 && cudaMalloc(&err, sizeof(int32_t)) != cudaSuccess) st = fail(BOLA_ERR_CUDA, "bola_dgemv_oz: out of memory");
  if (st == 0 && cudaMemsetAsync(err, 0, sizeof(int32_t), s) != cudaSuccess) st = BOLA_ERR_CUDA;
  if (st == 0) st = M.split(s, a, lda, nullptr);
  if (st == 0) st = M.product(s, (int)nrhs, x, ldx, b, ldb, out, ldo, err);
  int32_t herr = 0;
  if (st == 0 && cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, s) != cudaSuccess) st = BOLA_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess && st == 0) st = cuda_fail(cudaGetLastError(), "bola_dgemv_oz");
  if (err) cudaFree(err);
  M.release();
  if (st == 0 && herr != 0) st = fail(BOLA_ERR_CUDA, "bola_dgemv_oz: a bounded wait expired (code %d)", herr);
  return st;
}
