// calibrate.cu — FP64 throughput probe of the device the library runs on.
//
// The FP64 rate of a GB300 is far below its tensor rates and not a number to
// take from a datasheet, so roofline fractions of the FP64 kernels are stated
// against this measurement: eight
// independent register-resident DFMA chains per thread, four 256-thread
// blocks per SM, ~20 ms, timed with CUDA events.
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

}  // namespace
}  // namespace bola

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
