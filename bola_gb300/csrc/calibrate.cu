// calibrate.cu — probes of the device the library runs on: FP64 throughput
// (DFMA on the FP64 pipe, and DMMA on the tensor cores for comparison), the
// latency of one cluster exchange round, and a bounded-wait self-test.
//
// The FP64 rate of a GB300 is far below its tensor rates and not a number to
// take from a datasheet, so roofline fractions of the FP64 kernels are stated
// against this measurement: eight
// independent register-resident DFMA chains per thread, four 256-thread
// blocks per SM, ~20 ms, timed with CUDA events.
#include <cooperative_groups.h>

#include "common.cuh"
#include "sm100.cuh"

namespace bola {
namespace {

__global__ void dfma_probe(double *sink, int iters, double a, double b) {
  double acc[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = __fma_rn(acc[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s = __dadd_rn(s, acc[i]);
  if (s == 12345.678) sink[0] = s;  // keeps the loop alive; never true for these inputs
}

// The same measurement through the FP64 tensor-core instruction (DMMA,
// mma.sync m8n8k4 f64): eight independent accumulator tiles per warp.
__global__ void dmma_probe(double *sink, int iters, double a0, double b0) {
  const double a = a0 + threadIdx.x * 1e-12, b = b0 - threadIdx.x * 1e-12;
  double c[8][2];
#pragma unroll
  for (int i = 0; i < 8; ++i) c[i][0] = c[i][1] = 1e-3 * i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(c[i][0]), "+d"(c[i][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s = __dadd_rn(s, __dadd_rn(c[i][0], c[i][1]));
  if (s == 12345.678) sink[0] = s;  // keeps the loop alive; never true for these inputs
}

}  // namespace
}  // namespace bola

extern "C" int bola_measure_dmma_peak(double *gflops) {
  using namespace bola;
  if (gflops == nullptr) return -1;
  double *sink = nullptr;
  BOLA_TRY_CUDA(cudaMalloc(&sink, 64));
  const int sms = num_sms();
  const dim3 grid(4 * sms), block(256);
  const int iters = 2048;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dmma_probe<<<grid, block>>>(sink, 16, 1.0000001, 1e-9);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dmma_probe<<<grid, block>>>(sink, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaFree(sink);
      return cuda_fail(e, "dmma_probe");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  // 8 x 8 x 4 multiply-adds per warp instruction
  const double flops = 2.0 * 256.0 * 8.0 * iters * (double)grid.x * (block.x / 32);
  *gflops = flops / (best * 1e6);
  return 0;
}

extern "C" int bola_measure_fp64_peak(double *gflops) {
  using namespace bola;
  double *sink = nullptr;
  BOLA_TRY_CUDA(cudaMalloc(&sink, 64));
  const int sms = num_sms();
  const dim3 grid(4 * sms), block(256);
  const int iters = 6144;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dfma_probe<<<grid, block>>>(sink, 64, 1.0000001, 1e-9);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dfma_probe<<<grid, block>>>(sink, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaFree(sink);
      return cuda_fail(e, "dfma_probe");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  const double flops = 2.0 * 8.0 * iters * (double)grid.x * block.x;
  *gflops = flops / (best * 1e6);
  return 0;
}

// ---- bounded-wait self-test --------------------------------------------------
namespace bola {
namespace {

// Waits that can only end by giving up: an mbarrier with one expected arrival
// that never comes, and a flag that nothing sets.
__global__ void bounded_wait_selftest(int32_t *flag_err, uint32_t polls) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    sm100::mbar_init(&bar, 1);
    sm100::fence_mbar_init();
  }
  __syncthreads();
  const bool done = sm100::bounded_wait(&bar, 0u, polls);
  if (!done && threadIdx.x == 0) atomicOr(flag_err, 1);
  if (threadIdx.x == 0) {
    uint32_t p = 0;
    for (;;) {
      int v;
      asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(flag_err + 1) : "memory");
      if (v != 0) break;
      if (++p > polls) {
        atomicOr(flag_err, 2);
        break;
      }
      __nanosleep(64);
    }
  }
}

}  // namespace
}  // namespace bola

extern "C" int bola_selftest_bounded_waits(int32_t *flag_err, uint32_t polls, bola_stream_t stream) {
  using namespace bola;
  if (flag_err == nullptr) return -1;
  bounded_wait_selftest<<<1, 64, 0, (cudaStream_t)stream>>>(flag_err, polls);
  BOLA_CHECK_LAUNCH();
  return 0;
}

// ---- cluster exchange latency ------------------------------------------------
// The cluster panels of the mixed LU are latency-bound: their serial chain
// holds one all-to-all exchange per pivot group (per column for the FP64
// panel).  This probe times that exchange alone, as the floor a panel's time
// per group is stated against: per round, every CTA of a cluster copies
// `bytes` of its shared memory into a slot of every CTA (bulk copies that
// complete on the receiver's mbarrier), waits on its own mbarrier (bounded)
// and meets a CTA barrier.  Double-buffered slots, as in the panels.
namespace bola {
namespace {

namespace cgx = cooperative_groups;

__global__ void __launch_bounds__(256) exchange_probe(int rounds, uint32_t bytes, int32_t *err) {
  cgx::cluster_group cluster = cgx::this_cluster();
  const int C = (int)cluster.num_blocks(), cr = (int)cluster.block_rank();
  extern __shared__ __align__(128) unsigned char xp_raw[];  // [2][C][bytes] slots, then `bytes` of staging
  __shared__ uint64_t xbar[2];
  __shared__ int sfail;
  unsigned char *stage = xp_raw + 2 * (size_t)C * bytes;
  for (uint32_t i = threadIdx.x; i < bytes; i += blockDim.x) stage[i] = (unsigned char)i;
  if (threadIdx.x == 0) {
    sm100::mbar_init(&xbar[0], 1);
    sm100::mbar_init(&xbar[1], 1);
    sm100::fence_mbar_init();
    sfail = 0;
  }
  sm100::fence_proxy_async_smem();
  __syncthreads();
  cluster.sync();
  for (int r = 0; r < rounds; ++r) {
    const int par = r & 1;
    if (threadIdx.x == 0) sm100::mbar_arrive_expect_tx(&xbar[par], (uint32_t)C * bytes);
    if ((int)threadIdx.x < C) {
      const int d = threadIdx.x;
      const uint32_t dst = sm100::cluster_addr(xp_raw + ((size_t)par * C + cr) * bytes, d);
      asm volatile(
          "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
          "r"(sm100::smem_u32(stage)), "r"(bytes), "r"(sm100::cluster_addr(&xbar[par], d))
          : "memory");
      sm100::bulk_commit();
    }
    if (!sm100::bounded_wait(&xbar[par], (uint32_t)(r >> 1) & 1u)) sfail = 1;
    __syncthreads();
    if (sfail) {
      if (threadIdx.x == 0) atomicExch(err, 1);
      break;
    }
  }
  if ((int)threadIdx.x < C) sm100::bulk_wait_read0();
  cluster.sync();  // no CTA leaves while another may still copy into it
}

}  // namespace
}  // namespace bola

extern "C" int bola_measure_cluster_exchange(int csize, int bytes, double *us_per_round) {
  using namespace bola;
  if (csize < 1 || csize > 16) return -1;
  if (bytes < 16 || bytes > 8192 || (bytes & 15) != 0) return -2;
  if (us_per_round == nullptr) return -3;
  const size_t smem = (2 * (size_t)csize + 1) * (size_t)bytes;
  BOLA_TRY_CUDA(cudaFuncSetAttribute(exchange_probe, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  BOLA_TRY_CUDA(cudaFuncSetAttribute(exchange_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int32_t *err = nullptr;
  BOLA_TRY_CUDA(cudaMalloc(&err, sizeof(int32_t)));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)csize, 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = nullptr;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int st = 0;
  float ms[2] = {0.f, 0.f};
  const int rounds[2] = {200, 4200};  // the difference removes launch and set-up time
  if (cudaMemset(err, 0, sizeof(int32_t)) != cudaSuccess) st = fail(BOLA_ERR_CUDA, "exchange probe: memset");
  for (int k = 0; k < 2 && st == 0; ++k) {
    float best = 1e30f;
    for (int rep = 0; rep < 3 && st == 0; ++rep) {
      cudaEventRecord(e0);
      cudaError_t e = cudaLaunchKernelEx(&cfg, exchange_probe, rounds[k], (uint32_t)bytes, err);
      cudaEventRecord(e1);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) {
        st = cuda_fail(e, "exchange_probe");
        break;
      }
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      best = t < best ? t : best;
    }
    ms[k] = best;
  }
  int32_t herr = 0;
  if (st == 0 && cudaMemcpy(&herr, err, sizeof herr, cudaMemcpyDeviceToHost) != cudaSuccess)
    st = fail(BOLA_ERR_CUDA, "exchange probe: copy");
  if (st == 0 && herr != 0) st = fail(BOLA_ERR_CUDA, "exchange probe: a bounded wait expired");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(err);
  if (st == 0) *us_per_round = 1e3 * (double)(ms[1] - ms[0]) / (double)(rounds[1] - rounds[0]);
  return st;
}
