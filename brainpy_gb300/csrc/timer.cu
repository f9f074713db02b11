// timer.cu -- optional CUDA-event timing of each operator's dominant kernel.
//
// Off by default.  When enabled, every dominant-kernel launch is bracketed by a pair of
// CUDA events recorded on the launching stream; bp_timer_collect() synchronises those
// events and returns the summed kernel time.  Used by the benchmark to report the
// achieved bandwidth of the dominant kernel.
#include <mutex>
#include <vector>

#include "common.cuh"
#include "timer.cuh"

namespace bp {

namespace {
std::mutex g_mu;
bool g_on = false;
std::vector<cudaEvent_t> g_pool;  // pairs
size_t g_used = 0;
}  // namespace

bool timer_on() { return g_on; }

void timer_begin(cudaStream_t st, cudaEvent_t* stop_out) {
  *stop_out = nullptr;
  if (!g_on) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_used + 2 > g_pool.size()) {
    for (int k = 0; k < 256; ++k) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return;
      g_pool.push_back(e);
    }
  }
  cudaEventRecord(g_pool[g_used], st);
  *stop_out = g_pool[g_used + 1];
  g_used += 2;
}

void timer_end(cudaStream_t st, cudaEvent_t stop) {
  if (stop) cudaEventRecord(stop, st);
}

}  // namespace bp

extern "C" {

void bp_timer_enable(int32_t on) {
  std::lock_guard<std::mutex> lk(bp::g_mu);
  bp::g_on = on != 0;
  bp::g_used = 0;
}

bp_status bp_timer_collect(double* total_ms, int64_t* launches) {
  std::lock_guard<std::mutex> lk(bp::g_mu);
  double tot = 0.0;
  for (size_t k = 0; k + 1 < bp::g_used; k += 2) {
    BP_CUDA_TRY(cudaEventSynchronize(bp::g_pool[k + 1]));
    float ms = 0.f;
    BP_CUDA_TRY(cudaEventElapsedTime(&ms, bp::g_pool[k], bp::g_pool[k + 1]));
    tot += ms;
  }
  if (total_ms) *total_ms = tot;
  if (launches) *launches = (int64_t)(bp::g_used / 2);
  bp::g_used = 0;
  return BP_OK;
}

}  // extern "C"
