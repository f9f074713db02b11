// timer.cuh -- bracket a dominant-kernel launch with CUDA events (see timer.cu).
#pragma once
#include <cuda_runtime.h>

namespace bp {
bool timer_on();
void timer_begin(cudaStream_t st, cudaEvent_t* stop_out);
void timer_end(cudaStream_t st, cudaEvent_t stop);

struct ScopedKernelTimer {
  cudaStream_t st;
  cudaEvent_t stop;
  explicit ScopedKernelTimer(cudaStream_t s) : st(s), stop(nullptr) { timer_begin(st, &stop); }
  ~ScopedKernelTimer() { timer_end(st, stop); }
};
}  // namespace bp
