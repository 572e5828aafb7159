// profile.cuh — scope object that times the launches it encloses when the
// library's profiler is enabled (bola_profile_enable).
#pragma once

#include <cuda_runtime.h>

namespace bola {

bool profiling_on();

class ProfScope {
 public:
  // flops / bytes: algorithmic counts of the work the scope launches.
  // launches: kernels the scope enqueues.
  ProfScope(cudaStream_t s, const char *name, double flops = 0.0, double bytes = 0.0, int launches = 1);
  ~ProfScope();
  ProfScope(const ProfScope &) = delete;
  ProfScope &operator=(const ProfScope &) = delete;

 private:
  bool active_ = false;
  cudaStream_t s_ = nullptr;
  const char *name_ = nullptr;
  double flops_ = 0, bytes_ = 0;
  int launches_ = 1;
  cudaEvent_t a_ = nullptr, b_ = nullptr;
};

}  // namespace bola
