// profile.cu — per-routine device timers, the GPU counterpart of BOLA's
// `profiling` feature (src/profiling.rs:10-140: ScopedTimer + print_profile).
//
// When enabled, every kernel launch site records a CUDA event before and
// after the launch on the launching stream, tagged with a routine name and
// its algorithmic flop and byte counts.  bola_profile_read() synchronises on
// the recorded events and reports calls, device milliseconds, flops and bytes
// per name.  Disabled (the default), a scope costs one branch.
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "profile.cuh"

namespace bola {
namespace {

struct Rec {
  const char *name;
  cudaEvent_t a, b;
  double flops, bytes;
  int launches;
};
struct Agg {
  std::string name;
  int64_t calls = 0, launches = 0;
  double ms = 0, flops = 0, bytes = 0;
};

std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_pending;
std::vector<cudaEvent_t> g_pool;
std::vector<Agg> g_agg;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

Agg &agg_for(const char *name) {
  for (auto &a : g_agg)
    if (a.name == name) return a;
  g_agg.push_back(Agg{name});
  return g_agg.back();
}

// Folds finished records into the aggregates (caller holds the lock).
int drain() {
  for (auto &r : g_pending) {
    cudaError_t e = cudaEventSynchronize(r.b);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventSynchronize(profile)");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    Agg &a = agg_for(r.name);
    a.calls += 1;
    a.launches += r.launches;
    a.ms += ms;
    a.flops += r.flops;
    a.bytes += r.bytes;
    g_pool.push_back(r.a);
    g_pool.push_back(r.b);
  }
  g_pending.clear();
  return 0;
}

}  // namespace

bool profiling_on() { return g_on; }

ProfScope::ProfScope(cudaStream_t s, const char *name, double flops, double bytes, int launches) {
  if (!g_on) return;
  std::lock_guard<std::mutex> lk(g_mu);
  s_ = s;
  name_ = name;
  flops_ = flops;
  bytes_ = bytes;
  launches_ = launches;
  a_ = take_event();
  b_ = take_event();
  cudaEventRecord(a_, s);
  active_ = true;
}

ProfScope::~ProfScope() {
  if (!active_) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEventRecord(b_, s_);
  g_pending.push_back(Rec{name_, a_, b_, flops_, bytes_, launches_});
}

}  // namespace bola

using namespace bola;

extern "C" {

int bola_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  const int old = g_on ? 1 : 0;
  g_on = on != 0;
  return old;
}

int bola_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  const int r = drain();
  g_agg.clear();
  return r;
}

int bola_profile_count(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  const int r = drain();
  if (r) return r;
  return (int)g_agg.size();
}

int bola_profile_read(int index, char *name, int name_len, int64_t *calls, int64_t *launches, double *ms,
                      double *flops, double *bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  BOLA_TRY(drain());
  if (index < 0 || index >= (int)g_agg.size()) return -1;
  const Agg &a = g_agg[index];
  if (name && name_len > 0) {
    std::strncpy(name, a.name.c_str(), (size_t)name_len - 1);
    name[name_len - 1] = 0;
  }
  if (calls) *calls = a.calls;
  if (launches) *launches = a.launches;
  if (ms) *ms = a.ms;
  if (flops) *flops = a.flops;
  if (bytes) *bytes = a.bytes;
  return 0;
}

}  // extern "C"
