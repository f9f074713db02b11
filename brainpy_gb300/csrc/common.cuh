// common.cuh -- shared host/device helpers of libbpgpu (status handling, launch
// checks, warp utilities).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>

#include "../../include/bpgpu.h"

namespace bp {

constexpr int kNumSMs = 152;  // GB300; runtime code queries the device when it matters

// Per-thread message of the last failed call (read through bp_last_error()).
void set_error(const char* fmt, ...);
void clear_error();

// Returns BP_ECUDA (and records the message) if the last launch failed.
bp_status check_launch(const char* what);

inline cudaStream_t as_cuda(bp_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int device_sm_count();

#define BP_REQUIRE(cond, code, ...)    \
  do {                                 \
    if (!(cond)) {                     \
      ::bp::set_error(__VA_ARGS__);    \
      return code;                     \
    }                                  \
  } while (0)

#define BP_CUDA_TRY(expr)                                                          \
  do {                                                                             \
    cudaError_t e_ = (expr);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      ::bp::set_error("%s failed: %s", #expr, cudaGetErrorString(e_));             \
      return BP_ECUDA;                                                             \
    }                                                                              \
  } while (0)

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// event truth test for the three event encodings
__device__ __forceinline__ bool ev_on_f32(float e, int etype) {
  return etype == BP_EV_F32_POS ? (e > 0.0f) : (e != 0.0f);
}

}  // namespace bp
