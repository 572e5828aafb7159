// api.cu — library-wide state: error messages, SIMD-width setting, device info.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace bola {

namespace {
thread_local char g_msg[512] = "";
int g_lanes = 2;
}  // namespace

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof g_msg, fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(BOLA_ERR_CUDA, "%s failed: %s", what, cudaGetErrorString(e));
}

int lanes() { return g_lanes; }

int num_sms() {
  static thread_local int dev = -1, sms = 0;
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return 1;
  if (d != dev) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || v <= 0) v = 1;
    dev = d;
    sms = v;
  }
  return sms;
}

}  // namespace bola

extern "C" {

const char *bola_version(void) { return "bola_gb300 0.1.0 (sm_103a, BOLA 0.1.2 semantics)"; }

const char *bola_last_error(void) { return bola::g_msg; }

int bola_set_simd_lanes(int lanes) {
  if (lanes != 2 && lanes != 4) return -1;
  const int old = bola::g_lanes;
  bola::g_lanes = lanes;
  return old;
}

int bola_get_simd_lanes(void) { return bola::g_lanes; }

}  // extern "C"
