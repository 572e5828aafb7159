// dgemm.cu — FP64 GEMM with BOLA's rounding (src/gemm.rs:88-377), on DFMA.
//
// GB300's FP64 rate is ~1.2 TFLOP/s through DFMA (DMMA m8n8k4 measures 12% lower: bola_measure_dmma_peak),
// so this kernel is compute-bound at every shape BOLA's path produces: even a
// rank-32 update reads 16 B per 64 flop.  The design therefore spends its
// effort on keeping all 608 SM sub-partitions fed (tile size chosen per shape
// to minimise wave quantisation, split-K for skinny C) and on reproducing
// BOLA's accumulation order, which costs one extra DFMA per 64-deep chunk.
//
// Accumulation order, per element of C in BOLA's full 8x4 micro-tiles:
//   c = beta-scaled C;  for each K chunk of kc (64 in gemm, 32 in syrk):
//     acc = 0; for k in chunk: acc = fma(op(A)[i,k], op(B)[k,j], acc);
//     c = fma(alpha, acc, c)
// and in BOLA's partial edge tiles (rows >= m rounded down to 8, or columns
// >= n rounded down to 4): c = c + (alpha * op(B)[k,j]) * op(A)[i,k], unfused.
#include <cuda.h>

#include <mutex>

#include "common.cuh"

namespace bola {
namespace {

constexpr int KT = 16;  // K depth of one shared-memory stage (divides every kc)

__device__ __forceinline__ bool tri_keep(int tri, int64_t i, int64_t j) {
  if (tri == 0) return true;
  const int64_t bi = i >> 5, bj = j >> 5;
  return tri == 1 ? (bi < bj) : (bi > bj);
}

template <bool T>
__device__ __forceinline__ double op_a(const double *A, int64_t lda, int64_t i, int64_t k) {
  return T ? A[k + i * lda] : A[i + k * lda];
}
template <bool T>
__device__ __forceinline__ double op_b(const double *B, int64_t ldb, int64_t k, int64_t j) {
  return T ? B[j + k * ldb] : B[k + j * ldb];
}

// Main region [0, m8) x [0, n4).  PARTIAL: blockIdx.z owns a range of K
// chunks and writes each chunk's accumulator to P (split-K; the fold into C
// happens in chunk order in gemm_fold, so the result is unchanged).
template <int BM, int BN, int TM, int TN, bool TA, bool TB, bool PARTIAL>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_main(int64_t m8, int64_t n4, int64_t K, double alpha, const double *__restrict__ A, int64_t lda,
          const double *__restrict__ B, int64_t ldb, double beta, double *__restrict__ C, int64_t ldc,
          int kc, const int32_t *info, int tri, int64_t chunks_per_split, double *__restrict__ P) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int TX = BM / TM, TY = BN / TN;
  constexpr int AE = BM * KT / NT, BE = BN * KT / NT;
  static_assert((BM * KT) % NT == 0 && (BN * KT) % NT == 0, "tile/threads mismatch");
  __shared__ double As[2][KT][BM + 1];
  __shared__ double Bs[2][KT][BN + 1];

  if (stop_flag(info)) return;
  const int64_t i0 = (int64_t)blockIdx.x * BM, j0 = (int64_t)blockIdx.y * BN;
  if (tri == 1 && (i0 >> 5) >= ((j0 + BN - 1) >> 5)) return;
  if (tri == 2 && ((i0 + BM - 1) >> 5) <= (j0 >> 5)) return;
  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;

  const int64_t nchunks = (K + kc - 1) / kc;
  int64_t c_begin = 0, c_end = nchunks;
  if (PARTIAL) {
    c_begin = (int64_t)blockIdx.z * chunks_per_split;
    c_end = c_begin + chunks_per_split < nchunks ? c_begin + chunks_per_split : nchunks;
    if (c_begin >= c_end) return;
  }
  const int64_t kbeg = c_begin * kc;
  const int64_t kend = c_end * kc < K ? c_end * kc : K;

  double c[TM][TN], acc[TM][TN];
#pragma unroll
  for (int r = 0; r < TM; ++r)
#pragma unroll
    for (int q = 0; q < TN; ++q) {
      acc[r][q] = 0.0;
      c[r][q] = 0.0;
      if (!PARTIAL) {
        const int64_t gi = i0 + tx + TX * r, gj = j0 + ty + TY * q;
        if (gi < m8 && gj < n4 && beta != 0.0) {
          const double v = C[gi + gj * ldc];
          c[r][q] = (beta == 1.0) ? v : __dmul_rn(v, beta);
        }
      }
    }

  double ra[AE], rb[BE];
  auto gload = [&](int64_t k0) {
#pragma unroll
    for (int t = 0; t < AE; ++t) {
      const int e = tid + NT * t;
      const int ii = TA ? e / KT : e % BM;
      const int kk = TA ? e % KT : e / BM;
      const int64_t gi = i0 + ii, gk = k0 + kk;
      ra[t] = (gi < m8 && gk < kend) ? op_a<TA>(A, lda, gi, gk) : 0.0;
    }
#pragma unroll
    for (int t = 0; t < BE; ++t) {
      const int e = tid + NT * t;
      const int jj = TB ? e % BN : e / KT;
      const int kk = TB ? e / BN : e % KT;
      const int64_t gj = j0 + jj, gk = k0 + kk;
      rb[t] = (gj < n4 && gk < kend) ? op_b<TB>(B, ldb, gk, gj) : 0.0;
    }
  };
  auto sstore = [&](int buf) {
#pragma unroll
    for (int t = 0; t < AE; ++t) {
      const int e = tid + NT * t;
      const int ii = TA ? e / KT : e % BM;
      const int kk = TA ? e % KT : e / BM;
      As[buf][kk][ii] = ra[t];
    }
#pragma unroll
    for (int t = 0; t < BE; ++t) {
      const int e = tid + NT * t;
      const int jj = TB ? e % BN : e / KT;
      const int kk = TB ? e / BN : e % KT;
      Bs[buf][kk][jj] = rb[t];
    }
  };

  const int64_t nst = (kend - kbeg + KT - 1) / KT;
  if (nst > 0) {
    gload(kbeg);
    sstore(0);
  }
  __syncthreads();
  for (int64_t s = 0; s < nst; ++s) {
    const int64_t k0 = kbeg + s * KT;
    if (k0 % kc == 0) {
#pragma unroll
      for (int r = 0; r < TM; ++r)
#pragma unroll
        for (int q = 0; q < TN; ++q) acc[r][q] = 0.0;
    }
    if (s + 1 < nst) gload(k0 + KT);
    const int buf = (int)(s & 1);
#pragma unroll
    for (int kk = 0; kk < KT; ++kk) {
      double a[TM], b[TN];
#pragma unroll
      for (int r = 0; r < TM; ++r) a[r] = As[buf][kk][tx + TX * r];
#pragma unroll
      for (int q = 0; q < TN; ++q) b[q] = Bs[buf][kk][ty + TY * q];
#pragma unroll
      for (int r = 0; r < TM; ++r)
#pragma unroll
        for (int q = 0; q < TN; ++q) acc[r][q] = fused(a[r], b[q], acc[r][q]);
    }
    const bool chunk_end = ((k0 + KT) % kc == 0) || (s + 1 == nst);
    if (chunk_end) {
      if (PARTIAL) {
        const int64_t ch = k0 / kc;
        double *Pc = P + ch * (m8 * n4);
#pragma unroll
        for (int r = 0; r < TM; ++r)
#pragma unroll
          for (int q = 0; q < TN; ++q) {
            const int64_t gi = i0 + tx + TX * r, gj = j0 + ty + TY * q;
            if (gi < m8 && gj < n4) Pc[gi + gj * m8] = acc[r][q];
          }
      } else {
#pragma unroll
        for (int r = 0; r < TM; ++r)
#pragma unroll
          for (int q = 0; q < TN; ++q) c[r][q] = fused(alpha, acc[r][q], c[r][q]);
      }
    }
    if (s + 1 < nst) sstore(buf ^ 1);
    __syncthreads();
  }
  if constexpr (!PARTIAL) {
#pragma unroll
    for (int r = 0; r < TM; ++r)
#pragma unroll
      for (int q = 0; q < TN; ++q) {
        const int64_t gi = i0 + tx + TX * r, gj = j0 + ty + TY * q;
        if (gi < m8 && gj < n4 && tri_keep(tri, gi, gj)) C[gi + gj * ldc] = c[r][q];
      }
  }
}

// Fold split-K chunk accumulators into C in chunk order.
__global__ void gemm_fold(int64_t m8, int64_t n4, int64_t nchunks, double alpha, double beta,
                          const double *__restrict__ P, double *__restrict__ C, int64_t ldc,
                          const int32_t *info, int tri) {
  if (stop_flag(info)) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m8 * n4) return;
  const int64_t i = e % m8, j = e / m8;
  if (!tri_keep(tri, i, j)) return;
  double c = 0.0;
  if (beta != 0.0) {
    c = C[i + j * ldc];
    if (beta != 1.0) c = __dmul_rn(c, beta);
  }
  for (int64_t ch = 0; ch < nchunks; ++ch) c = fused(alpha, P[ch * (m8 * n4) + e], c);
  C[i + j * ldc] = c;
}

// BOLA's edge tiles (add_scalar_kernel, src/gemm.rs:357-377): unfused
// c += (alpha * b) * a over all k in order.
template <bool TA, bool TB>
__global__ void gemm_edge(int64_t m, int64_t n, int64_t m8, int64_t n4, int64_t K, double alpha,
                          const double *__restrict__ A, int64_t lda, const double *__restrict__ B,
                          int64_t ldb, double beta, double *__restrict__ C, int64_t ldc,
                          const int32_t *info, int tri) {
  if (stop_flag(info)) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t e1 = (m - m8) * n, e2 = m8 * (n - n4);
  if (e >= e1 + e2) return;
  int64_t i, j;
  if (e < e1) {
    i = m8 + e % (m - m8);
    j = e / (m - m8);
  } else {
    const int64_t f = e - e1;
    i = f % m8;
    j = n4 + f / m8;
  }
  if (!tri_keep(tri, i, j)) return;
  double c = 0.0;
  if (beta != 0.0) {
    c = C[i + j * ldc];
    if (beta != 1.0) c = __dmul_rn(c, beta);
  }
  for (int64_t k = 0; k < K; ++k) {
    const double t = __dmul_rn(alpha, op_b<TB>(B, ldb, k, j));
    c = add_prod(c, t, op_a<TA>(A, lda, i, k));
  }
  C[i + j * ldc] = c;
}

struct Tile {
  int bm, bn;
};

template <int BM, int BN, int TM, int TN, bool TA, bool TB, bool PARTIAL>
void launch_main(cudaStream_t s, dim3 grid, int64_t m8, int64_t n4, int64_t K, double alpha,
                 const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                 int64_t ldc, int kc, const int32_t *info, int tri, int64_t cps, double *P) {
  gemm_main<BM, BN, TM, TN, TA, TB, PARTIAL><<<grid, (BM / TM) * (BN / TN), 0, s>>>(
      m8, n4, K, alpha, A, lda, B, ldb, beta, C, ldc, kc, info, tri, cps, P);
}

template <bool TA, bool TB>
void launch_tile(Tile t, bool partial, cudaStream_t s, dim3 grid, int64_t m8, int64_t n4, int64_t K,
                 double alpha, const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                 double *C, int64_t ldc, int kc, const int32_t *info, int tri, int64_t cps, double *P) {
#define BOLA_LM(bm, bn, tm, tn)                                                                                    \
  (partial ? launch_main<bm, bn, tm, tn, TA, TB, true>(s, grid, m8, n4, K, alpha, A, lda, B, ldb, beta, C, ldc, kc, \
                                                     info, tri, cps, P)                                            \
           : launch_main<bm, bn, tm, tn, TA, TB, false>(s, grid, m8, n4, K, alpha, A, lda, B, ldb, beta, C, ldc,    \
                                                      kc, info, tri, cps, P))
  if (t.bm == 64 && t.bn == 64) BOLA_LM(64, 64, 4, 4);
  else if (t.bm == 64 && t.bn == 32) BOLA_LM(64, 32, 4, 2);
  else if (t.bm == 32 && t.bn == 64) BOLA_LM(32, 64, 2, 4);
  else if (t.bm == 64 && t.bn == 16) BOLA_LM(64, 16, 4, 1);
  else BOLA_LM(32, 32, 2, 2);
#undef BOLA_LM
}

// Pick the tile whose most-loaded SM carries the least tile area (ties go to
// the larger tile).
Tile choose_tile(int64_t m8, int64_t n4, int sms) {
  // 64x16 serves skinny outputs such as 16 right-hand sides
  const Tile cands[5] = {{64, 64}, {64, 32}, {32, 64}, {32, 32}, {64, 16}};
  Tile best = cands[0];
  double best_cost = 1e300;
  for (const Tile &t : cands) {
    const int64_t T = cdiv(m8, t.bm) * cdiv(n4, t.bn);
    const double cost = (double)cdiv(T, sms) * t.bm * t.bn;
    if (cost < best_cost * 0.999) {
      best_cost = cost;
      best = t;
    }
  }
  return best;
}

}  // namespace

namespace {

// The exact DGEMM.  Split-K partial sums go to stream-ordered temporary
// memory, or, when `fixed` is given, to that caller-provided device buffer of
// `fixed_bytes` (a shape whose partial sums do not fit is rejected before
// anything is launched).
int dgemm_body(cudaStream_t s, char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
               const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
               int64_t ldc, int kc, const int32_t *info, int tri, double *fixed, size_t fixed_bytes) {
  if (m <= 0 || n <= 0) return 0;
  const bool TA = upc(ta) != 'N', TB = upc(tb) != 'N';
  const int64_t K = (alpha == 0.0 || k < 0) ? 0 : k;  // alpha == 0: only the beta pass
  const int64_t m8 = (m / 8) * 8, n4 = (n / 4) * 4;
  const int sms = num_sms();
  if (m8 > 0 && n4 > 0) {
    Tile t = choose_tile(m8, n4, sms);
    const int64_t nchunks = (K + kc - 1) / kc;
    int64_t tiles = cdiv(m8, t.bm) * cdiv(n4, t.bn);
    bool partial = false;
    int64_t cps = 0, nsplit = 1;
    if (tiles < sms && nchunks >= 2) {
      nsplit = imin(nchunks, cdiv(2 * (int64_t)sms, tiles));
      cps = cdiv(nchunks, nsplit);
      nsplit = cdiv(nchunks, cps);
      const double bytes = 8.0 * (double)nchunks * (double)m8 * (double)n4;
      partial = nsplit >= 2 && bytes <= (1u << 30);
      if (partial && fixed != nullptr && bytes > (double)fixed_bytes)
        return fail(BOLA_ERR_UNSUPPORTED,
                    "bola_dgemm_noalloc: this shape needs %.0f bytes of split-K scratch, the static scratch "
                    "holds %zu bytes (%lld chunks x %lld x %lld doubles); use bola_dgemm",
                    bytes, fixed_bytes, (long long)nchunks, (long long)m8, (long long)n4);
    }
    ProfScope prof(s, "dgemm", 2.0 * (double)m8 * (double)n4 * (double)K,
                   8.0 * ((double)m8 * K + (double)K * n4 + 2.0 * (double)m8 * n4), partial ? 2 : 1);
    if (partial) {
      // Every partial sum the fold reads is written by this call's partial
      // pass, so a reused buffer (the fixed one) needs no clearing.
      Scratch Ps;
      if (fixed == nullptr) BOLA_TRY(Ps.alloc((size_t)(8 * nchunks * m8 * n4), s));
      double *P = fixed != nullptr ? fixed : Ps.as<double>();
      dim3 grid((unsigned)cdiv(m8, t.bm), (unsigned)cdiv(n4, t.bn), (unsigned)nsplit);
#define BOLA_LT(a, b)                                                                            \
  launch_tile<a, b>(t, true, s, grid, m8, n4, K, alpha, A, lda, B, ldb, beta, C, ldc, kc, info, tri, \
                    cps, P)
      if (!TA && !TB) BOLA_LT(false, false);
      else if (!TA && TB) BOLA_LT(false, true);
      else if (TA && !TB) BOLA_LT(true, false);
      else BOLA_LT(true, true);
#undef BOLA_LT
      BOLA_CHECK_LAUNCH();
      const int64_t tot = m8 * n4;
      gemm_fold<<<(unsigned)cdiv(tot, 256), 256, 0, s>>>(m8, n4, nchunks, alpha, beta, P, C, ldc, info, tri);
      BOLA_CHECK_LAUNCH();
    } else {
      dim3 grid((unsigned)cdiv(m8, t.bm), (unsigned)cdiv(n4, t.bn), 1);
#define BOLA_LT(a, b) \
  launch_tile<a, b>(t, false, s, grid, m8, n4, K, alpha, A, lda, B, ldb, beta, C, ldc, kc, info, tri, 0, nullptr)
      if (!TA && !TB) BOLA_LT(false, false);
      else if (!TA && TB) BOLA_LT(false, true);
      else if (TA && !TB) BOLA_LT(true, false);
      else BOLA_LT(true, true);
#undef BOLA_LT
      BOLA_CHECK_LAUNCH();
    }
  }
  const int64_t ne = (m - m8) * n + m8 * (n - n4);
  if (ne > 0) {
    ProfScope prof(s, "dgemm_edge", 2.0 * (double)ne * (double)K);
    const unsigned g = (unsigned)cdiv(ne, 128);
#define BOLA_LE(a, b) \
  gemm_edge<a, b><<<g, 128, 0, s>>>(m, n, m8, n4, K, alpha, A, lda, B, ldb, beta, C, ldc, info, tri)
    if (!TA && !TB) BOLA_LE(false, false);
    else if (!TA && TB) BOLA_LE(false, true);
    else if (TA && !TB) BOLA_LE(true, false);
    else BOLA_LE(true, true);
#undef BOLA_LE
    BOLA_CHECK_LAUNCH();
  }
  return 0;
}

}  // namespace

int dgemm_exact(cudaStream_t s, char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
                const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                int64_t ldc, int kc, const int32_t *info, int tri) {
  return dgemm_body(s, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, kc, info, tri, nullptr, 0);
}

}  // namespace bola

extern "C" int bola_dgemm(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
                          const double *a, int64_t lda, const double *b, int64_t ldb, double beta,
                          double *c, int64_t ldc, bola_stream_t stream) {
  // BOLA validates nothing beyond the empty-matrix exit (src/gemm.rs:106-108);
  // negative sizes and leading dimensions that cannot address the operands are
  // rejected here because a GPU out-of-bounds access would not stay local.
  if (m < 0) return -3;
  if (n < 0) return -4;
  if (k < 0) return -5;
  if (m == 0 || n == 0) return 0;
  const bool ta = bola::upc(transa) != 'N', tb = bola::upc(transb) != 'N';
  if (k > 0 && alpha != 0.0 && lda < bola::imax(1, ta ? k : m)) return -8;
  if (k > 0 && alpha != 0.0 && ldb < bola::imax(1, tb ? n : k)) return -10;
  if (ldc < bola::imax(1, m)) return -13;
  return bola::dgemm_exact((cudaStream_t)stream, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta,
                           c, ldc, 64, nullptr, 0);
}

// ---- allocation-free DGEMM ---------------------------------------------------
// For callers that may not allocate device memory (see bola_dgemm_noalloc in
// include/bola_gb300.h).  When the output is too small to keep every SM busy,
// bola_dgemm splits K and parks one partial accumulator per K chunk in
// stream-ordered temporary memory; this variant runs the same body (the same
// tile, split and launches, so its results are bola_dgemm's bit for bit) with
// the partial sums parked in a fixed array that lives in the library's own
// device image instead.

namespace bola {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;

// One copy per device that loads this library, held until the process exits.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchBytes / sizeof(double)];

std::mutex g_noalloc_mu;
struct NoAllocSlot {
  unsigned long long ctx_id = 0;  // the context the address belongs to (0: none yet)
  double *ptr = nullptr;
};
NoAllocSlot g_noalloc_slot[kMaxDevices];

// Unique id of the calling thread's current context (0 if none or unknown).
// The driver functions are reached through the runtime's entry-point query,
// so the library does not link the driver library directly.
unsigned long long current_context_id() {
  using GetCurrentFn = CUresult (*)(CUcontext *);
  using GetIdFn = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(p);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current == nullptr || get_id == nullptr || get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr ||
      get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of the scratch array in the current context.  The host-side
// symbol is only a stand-in, so the address is looked up with the device
// current and cached per device together with the context's unique id: a
// device reset destroys the context and unloads the module, and the next
// context may place the array elsewhere, so a new id means a new lookup.
int noalloc_scratch(double **out) {
  int dev = 0;
  BOLA_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(BOLA_ERR_UNSUPPORTED, "bola_dgemm_noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocSlot &slot = g_noalloc_slot[dev];
  unsigned long long id = current_context_id();
  if (slot.ptr == nullptr || id == 0 || slot.ctx_id != id) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    if (id == 0) id = current_context_id();  // the lookup initialised the context
    slot.ptr = static_cast<double *>(p);
    slot.ctx_id = id;
  }
  *out = slot.ptr;
  return 0;
}

}  // namespace
}  // namespace bola

extern "C" int bola_dgemm_noalloc(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
                                  const double *a, int64_t lda, const double *b, int64_t ldb, double beta,
                                  double *c, int64_t ldc, bola_stream_t stream) {
  using namespace bola;
  if (m < 0) return -3;
  if (n < 0) return -4;
  if (k < 0) return -5;
  if (m == 0 || n == 0) return 0;
  const bool ta = upc(transa) != 'N', tb = upc(transb) != 'N';
  if (k > 0 && alpha != 0.0 && lda < imax(1, ta ? k : m)) return -8;
  if (k > 0 && alpha != 0.0 && ldb < imax(1, tb ? n : k)) return -10;
  if (ldc < imax(1, m)) return -13;
  double *P = nullptr;
  BOLA_TRY(noalloc_scratch(&P));
  return dgemm_body((cudaStream_t)stream, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 64, nullptr,
                    0, P, kNoAllocScratchBytes);
}
