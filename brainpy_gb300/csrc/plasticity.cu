// plasticity.cu -- the CSR layers' STDP weight updates, event-driven.
//
// bp_csr_on_pre_update: for every pre-synaptic row i with spike[i], each synapse k of the row
//   becomes min(max(w[k] + trace[indices[k]], w_min), w_max).
// bp_csc_on_post_update: for every post-synaptic column i with spike[i], each entry k of the
//   column updates synapse w_ids[k] with trace[pre_ids[k]] the same way.
// Reference: brainpy/_src/dnn/linear.py:650-698 (_cpu_csr_on_pre_update, _cpu_csc_on_pre_update),
// which copy the weights and loop serially over all rows.  Here the spiking rows (columns) are
// compacted first, then warps share them out: a spiking row streams its index/weight run
// coalesced and gathers the trace.  Every synapse belongs to one row (column), so the updates
// never collide.  The clip keeps NaN, as numpy's minimum/maximum do.
#include "common.cuh"
#include "compact.cuh"
#include "timer.cuh"

namespace bp {

__device__ __forceinline__ float clip_np(float x, float lo, float hi) {
  x = x < lo ? lo : x;
  return x > hi ? hi : x;
}


// The spiking rows (columns) come from the unordered compaction; each warp then takes list
// entries a = warp, warp + W, ... and walks the row's synapses 256 at a time, 8 per lane with
// all loads of a round issued before the first store (the latency chain index -> trace/weight
// -> store is otherwise paid per 32 synapses).
constexpr int kStdpUnroll = 8;

// Row bounds of list entry a (clamped to [0, nnz]); a past the count gives an empty range.
template <typename IdxT>
__device__ __forceinline__ void stdp_bounds(const IdxT* __restrict__ indptr, const int32_t* __restrict__ list,
                                            int64_t a, int64_t cnt, int64_t nnz, int64_t& b, int64_t& e) {
  b = e = 0;
  if (a < cnt) {
    const int64_t r = __ldg(list + a);
    b = (int64_t)indptr[r];
    e = (int64_t)indptr[r + 1];
    b = b < 0 ? 0 : (b > nnz ? nnz : b);
    e = e < b ? b : (e > nnz ? nnz : e);
  }
}

template <typename IdxT>
__global__ void __launch_bounds__(256, 8) csr_on_pre_kernel(float* __restrict__ w, const IdxT* __restrict__ indices,
                                                            const IdxT* __restrict__ indptr, int64_t nnz, int64_t n,
                                                            const int32_t* __restrict__ list,
                                                            const int32_t* __restrict__ count,
                                                            const float* __restrict__ trace, float lo, float hi) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t cnt = *count;
  int64_t a = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int64_t nb, ne;  // bounds of the warp's next row, loaded while the current one is updated
  stdp_bounds(indptr, list, a, cnt, nnz, nb, ne);
  for (; a < cnt; a += nwarps) {
    const int64_t b = nb, e = ne;
    stdp_bounds(indptr, list, a + nwarps, cnt, nnz, nb, ne);
    for (int64_t k0 = b + lane; k0 < e; k0 += 32 * kStdpUnroll) {
      int64_t c[kStdpUnroll];
      float x[kStdpUnroll];
#pragma unroll
      for (int u = 0; u < kStdpUnroll; ++u) {
        const int64_t k = k0 + 32 * u;
        c[u] = k < e ? (int64_t)indices[k] : -1;
      }
#pragma unroll
      for (int u = 0; u < kStdpUnroll; ++u) {
        const bool ok = (uint64_t)c[u] < (uint64_t)n;
        x[u] = ok ? __fadd_rn(w[k0 + 32 * u], __ldg(trace + c[u])) : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < kStdpUnroll; ++u)
        if ((uint64_t)c[u] < (uint64_t)n) w[k0 + 32 * u] = clip_np(x[u], lo, hi);
    }
  }
}

template <typename IdxT>
__global__ void __launch_bounds__(256) csc_on_post_kernel(float* __restrict__ w, const IdxT* __restrict__ pre_ids,
                                                          const IdxT* __restrict__ indptr,
                                                          const IdxT* __restrict__ w_ids, int64_t nnz, int64_t m,
                                                          const int32_t* __restrict__ list,
                                                          const int32_t* __restrict__ count,
                                                          const float* __restrict__ trace, float lo, float hi) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t cnt = *count;
  int64_t a = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int64_t nb, ne;
  stdp_bounds(indptr, list, a, cnt, nnz, nb, ne);
  for (; a < cnt; a += nwarps) {
    const int64_t b = nb, e = ne;
    stdp_bounds(indptr, list, a + nwarps, cnt, nnz, nb, ne);
    for (int64_t k0 = b + lane; k0 < e; k0 += 32 * kStdpUnroll) {
      int64_t l[kStdpUnroll], j[kStdpUnroll];
      float x[kStdpUnroll];
#pragma unroll
      for (int u = 0; u < kStdpUnroll; ++u) {
        const int64_t k = k0 + 32 * u;
        l[u] = k < e ? (int64_t)w_ids[k] : -1;
        j[u] = k < e ? (int64_t)pre_ids[k] : -1;
      }
#pragma unroll
      for (int u = 0; u < kStdpUnroll; ++u) {
        const bool ok = (uint64_t)l[u] < (uint64_t)nnz && (uint64_t)j[u] < (uint64_t)m;
        x[u] = ok ? __fadd_rn(w[l[u]], __ldg(trace + j[u])) : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < kStdpUnroll; ++u)
        if ((uint64_t)l[u] < (uint64_t)nnz && (uint64_t)j[u] < (uint64_t)m) w[l[u]] = clip_np(x[u], lo, hi);
    }
  }
}

// a grid of exactly the CTAs that fit at once (the warps stride over the spiking rows)
template <typename K>
static int resident_grid(K kfn) {
  static int cache[64] = {0};  // per device: CTAs of 256 threads per SM
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (cache[dev] == 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, 256, 0) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      per_sm = 4;
    }
    cache[dev] = per_sm;
  }
  return device_sm_count() * cache[dev];
}

static size_t stdp_list_bytes(int64_t rows) { return align_up(sizeof(int32_t) * (size_t)(rows > 0 ? rows : 1), 256); }

// w_out = w_in (unless the same buffer), before the update
static bp_status copy_weights(const float* w_in, float* w_out, int64_t nnz, cudaStream_t st) {
  if (w_in != w_out && nnz > 0)
    BP_CUDA_TRY(cudaMemcpyAsync(w_out, w_in, sizeof(float) * (size_t)nnz, cudaMemcpyDeviceToDevice, st));
  return BP_OK;
}

// compaction of the spike vector into the workspace: list (rows entries), then the count
static bp_status stdp_compact(const void* spike, bp_etype et, int64_t rows, void* ws, int32_t*& list,
                              int32_t*& count, cudaStream_t st) {
  list = static_cast<int32_t*>(ws);
  count = reinterpret_cast<int32_t*>(static_cast<char*>(ws) + stdp_list_bytes(rows));
  BP_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(int32_t), st));
  return compact_events(spike, et, rows, list, count, st);
}

}  // namespace bp

using namespace bp;

extern "C" {

size_t bp_stdp_workspace_size(int64_t rows) { return stdp_list_bytes(rows) + 256; }

bp_status bp_csr_on_pre_update(const float* w_in, float* w_out, const void* indices, const void* indptr,
                               bp_itype itype, int64_t nnz, int64_t m, int64_t n, const void* spike, bp_etype etype,
                               const float* trace, float w_min, float w_max, void* workspace, size_t workspace_bytes,
                               bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(m >= 0 && n >= 0 && nnz >= 0, BP_EINVAL, "csr_on_pre_update: negative size");
  BP_REQUIRE(m <= INT32_MAX, BP_ENOTSUP, "csr_on_pre_update: more than 2^31 rows");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "csr_on_pre_update: bad index type %d", (int)itype);
  BP_REQUIRE(etype == BP_EV_BOOL || etype == BP_EV_F32_NZ || etype == BP_EV_F32_POS, BP_EDTYPE,
             "csr_on_pre_update: bad spike type %d", (int)etype);
  if (nnz == 0) return BP_OK;
  BP_REQUIRE(w_in && w_out, BP_EINVAL, "csr_on_pre_update: null weights");
  bp_status s = copy_weights(w_in, w_out, nnz, st);
  if (s != BP_OK || m == 0) return s;
  BP_REQUIRE(indices && indptr && spike && (trace || n == 0), BP_EINVAL, "csr_on_pre_update: null pointer");
  BP_REQUIRE(workspace && workspace_bytes >= bp_stdp_workspace_size(m), BP_ENOMEM,
             "csr_on_pre_update: workspace %zu < %zu", workspace_bytes, bp_stdp_workspace_size(m));
  ScopedKernelTimer tk(st);
  int32_t *list = nullptr, *count = nullptr;
  s = stdp_compact(spike, etype == BP_EV_BOOL ? BP_EV_BOOL : BP_EV_F32_NZ, m, workspace, list, count, st);
  if (s != BP_OK) return s;
  if (itype == BP_I32)
    csr_on_pre_kernel<int32_t><<<resident_grid(csr_on_pre_kernel<int32_t>), 256, 0, st>>>(w_out, static_cast<const int32_t*>(indices),
                                                  static_cast<const int32_t*>(indptr), nnz, n, list, count, trace,
                                                  w_min, w_max);
  else
    csr_on_pre_kernel<int64_t><<<resident_grid(csr_on_pre_kernel<int64_t>), 256, 0, st>>>(w_out, static_cast<const int64_t*>(indices),
                                                  static_cast<const int64_t*>(indptr), nnz, n, list, count, trace,
                                                  w_min, w_max);
  return check_launch("csr_on_pre_kernel");
}

bp_status bp_csc_on_post_update(const float* w_in, float* w_out, const void* pre_ids, const void* indptr,
                                const void* w_ids, bp_itype itype, int64_t nnz, int64_t n, int64_t m,
                                const void* spike, bp_etype etype, const float* trace, float w_min, float w_max,
                                void* workspace, size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(m >= 0 && n >= 0 && nnz >= 0, BP_EINVAL, "csc_on_post_update: negative size");
  BP_REQUIRE(n <= INT32_MAX, BP_ENOTSUP, "csc_on_post_update: more than 2^31 columns");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "csc_on_post_update: bad index type %d", (int)itype);
  BP_REQUIRE(etype == BP_EV_BOOL || etype == BP_EV_F32_NZ || etype == BP_EV_F32_POS, BP_EDTYPE,
             "csc_on_post_update: bad spike type %d", (int)etype);
  if (nnz == 0) return BP_OK;
  BP_REQUIRE(w_in && w_out, BP_EINVAL, "csc_on_post_update: null weights");
  bp_status s = copy_weights(w_in, w_out, nnz, st);
  if (s != BP_OK || n == 0) return s;
  BP_REQUIRE(pre_ids && indptr && w_ids && spike && (trace || m == 0), BP_EINVAL, "csc_on_post_update: null pointer");
  BP_REQUIRE(workspace && workspace_bytes >= bp_stdp_workspace_size(n), BP_ENOMEM,
             "csc_on_post_update: workspace %zu < %zu", workspace_bytes, bp_stdp_workspace_size(n));
  ScopedKernelTimer tk(st);
  int32_t *list = nullptr, *count = nullptr;
  s = stdp_compact(spike, etype == BP_EV_BOOL ? BP_EV_BOOL : BP_EV_F32_NZ, n, workspace, list, count, st);
  if (s != BP_OK) return s;
  if (itype == BP_I32)
    csc_on_post_kernel<int32_t><<<resident_grid(csc_on_post_kernel<int32_t>), 256, 0, st>>>(w_out, static_cast<const int32_t*>(pre_ids),
                                                   static_cast<const int32_t*>(indptr),
                                                   static_cast<const int32_t*>(w_ids), nnz, m, list, count, trace,
                                                   w_min, w_max);
  else
    csc_on_post_kernel<int64_t><<<resident_grid(csc_on_post_kernel<int64_t>), 256, 0, st>>>(w_out, static_cast<const int64_t*>(pre_ids),
                                                   static_cast<const int64_t*>(indptr),
                                                   static_cast<const int64_t*>(w_ids), nnz, m, list, count, trace,
                                                   w_min, w_max);
  return check_launch("csc_on_post_kernel");
}

}  // extern "C"
