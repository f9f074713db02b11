// compact.cuh -- spike-vector compaction (warp ballot / popc) shared by the
// event operators.
#pragma once

#include "common.cuh"

namespace bp {

// Loads up to 16 consecutive events starting at `base` and returns a bit mask of the
// active ones (bit k <-> element base + k).  `vec_ok` says the pointer is 16-byte aligned.
template <int ET>
__device__ __forceinline__ uint32_t load_event_mask16(const void* events, int64_t base, int64_t n, bool vec_ok) {
  uint32_t mask = 0;
  if (ET == BP_EV_BOOL) {
    const uint8_t* ev = static_cast<const uint8_t*>(events);
    if (vec_ok && base + 16 <= n) {
      uint4 v = __ldg(reinterpret_cast<const uint4*>(ev + base));
      uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int b = 0; b < 4; ++b)
          if ((w[q] >> (8 * b)) & 0xffu) mask |= 1u << (4 * q + b);
    } else {
      for (int k = 0; k < 16 && base + k < n; ++k)
        if (ev[base + k]) mask |= 1u << k;
    }
  } else {
    const float* ev = static_cast<const float*>(events);
    if (vec_ok && base + 16 <= n) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float4 v = __ldg(reinterpret_cast<const float4*>(ev + base) + q);
        if (ev_on_f32(v.x, ET)) mask |= 1u << (4 * q + 0);
        if (ev_on_f32(v.y, ET)) mask |= 1u << (4 * q + 1);
        if (ev_on_f32(v.z, ET)) mask |= 1u << (4 * q + 2);
        if (ev_on_f32(v.w, ET)) mask |= 1u << (4 * q + 3);
      }
    } else {
      for (int k = 0; k < 16 && base + k < n; ++k)
        if (ev_on_f32(ev[base + k], ET)) mask |= 1u << k;
    }
  }
  return mask;
}

// Unordered compaction: appends the indices of active events to list[], count in *count
// (which must be zero on entry).  One global atomic per warp.
template <int ET>
__global__ void __launch_bounds__(256) compact_unordered_kernel(const void* __restrict__ events, int64_t n,
                                                                int32_t* __restrict__ list,
                                                                int32_t* __restrict__ count) {
  const bool vec_ok = ((reinterpret_cast<uintptr_t>(events) & 15u) == 0);
  const int lane = lane_id();
  const int64_t per_iter = (int64_t)gridDim.x * blockDim.x * 16;
  for (int64_t chunk = ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31)) * 16; chunk < n; chunk += per_iter) {
    const int64_t base = chunk + (int64_t)lane * 16;
    uint32_t mask = base < n ? load_event_mask16<ET>(events, base, n, vec_ok) : 0u;
    int c = __popc(mask);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    int total = __shfl_sync(0xffffffffu, incl, 31);
    int wbase = 0;
    if (lane == 31 && total) wbase = atomicAdd(count, total);
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    int pos = wbase + incl - c;
    while (mask) {
      int k = __ffs(mask) - 1;
      mask &= mask - 1;
      list[pos++] = (int32_t)(base + k);
    }
  }
}

// Host side (event_csrmv.cu): launches compact_unordered_kernel for the event type; *count must
// be zero on entry.
bp_status compact_events(const void* events, bp_etype et, int64_t m, int32_t* list, int32_t* count,
                         cudaStream_t st);

}  // namespace bp
