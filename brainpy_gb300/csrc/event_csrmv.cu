// event_csrmv.cu -- event.info and event.csrmv on plain CSR.
//
// event.csrmv, transpose=1 (the event-driven form): the spike vector is compacted to
// the list of active rows, then one warp per active row streams the row's column
// indices and adds into the output.  Homogeneous weights accumulate exact uint32
// event counts (out = count * w at the end); heterogeneous weights accumulate float32.
// transpose=0: one warp per row gathers the event flags of its columns.
//
// Reference semantics: brainpy/_src/math/event/_csr_matvec.py:321-412 (Numba CPU),
// brainpy/_src/math/event/_csr_matvec_taichi.py:158-312 (Taichi GPU: warp per row,
// global atomics).
#include <cooperative_groups.h>

#include "common.cuh"
#include "compact.cuh"
#include "timer.cuh"

namespace cg = cooperative_groups;

namespace bp {

// ---------------------------------------------------------------------------
// ordered compaction (event.info)
// ---------------------------------------------------------------------------
constexpr int kInfoThreads = 256;
constexpr int kInfoChunk = kInfoThreads * 16;  // events per block

template <int ET>
__global__ void __launch_bounds__(kInfoThreads) info_count_kernel(const void* __restrict__ events, int64_t n,
                                                                  int32_t* __restrict__ block_counts) {
  const bool vec_ok = ((reinterpret_cast<uintptr_t>(events) & 15u) == 0);
  int64_t base = (int64_t)blockIdx.x * kInfoChunk + (int64_t)threadIdx.x * 16;
  uint32_t mask = base < n ? load_event_mask16<ET>(events, base, n, vec_ok) : 0u;
  int c = __popc(mask);
  __shared__ int warp_tot[kInfoThreads / 32];
  c = warp_sum(c);
  if (lane_id() == 0) warp_tot[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kInfoThreads / 32; ++w) s += warp_tot[w];
    block_counts[blockIdx.x] = s;
  }
}

// Exclusive scan of block_counts in place (single block); total -> *num.
__global__ void __launch_bounds__(1024) info_scan_kernel(int32_t* __restrict__ block_counts, int nb,
                                                         int32_t* __restrict__ num) {
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    int i = base + threadIdx.x;
    int v = i < nb ? block_counts[i] : 0;
    int incl = v;
    const int lane = lane_id(), w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
      int t = warp_tot[lane];
      int ti = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, ti, o);
        if (lane >= o) ti += u;
      }
      warp_tot[lane] = ti - t;
    }
    __syncthreads();
    int excl = carry + warp_tot[w] + incl - v;
    if (i < nb) block_counts[i] = excl;
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *num = carry;
}

template <int ET>
__global__ void __launch_bounds__(kInfoThreads) info_write_kernel(const void* __restrict__ events, int64_t n,
                                                                  const int32_t* __restrict__ block_offsets,
                                                                  const int32_t* __restrict__ num,
                                                                  int32_t* __restrict__ ids) {
  const bool vec_ok = ((reinterpret_cast<uintptr_t>(events) & 15u) == 0);
  const int64_t blk0 = (int64_t)blockIdx.x * kInfoChunk;
  int64_t base = blk0 + (int64_t)threadIdx.x * 16;
  uint32_t mask = base < n ? load_event_mask16<ET>(events, base, n, vec_ok) : 0u;
  int c = __popc(mask);
  const int lane = lane_id(), w = threadIdx.x >> 5;
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  __shared__ int warp_tot[kInfoThreads / 32];
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  int wpre = 0;
  for (int k = 0; k < w; ++k) wpre += warp_tot[k];
  int pos = block_offsets[blockIdx.x] + wpre + incl - c;
  while (mask) {
    int k = __ffs(mask) - 1;
    mask &= mask - 1;
    ids[pos++] = (int32_t)(base + k);
  }
  // pad: output positions of this block's range that lie beyond the total count
  const int total = *num;
  for (int64_t p = blk0 + threadIdx.x; p < blk0 + kInfoChunk && p < n; p += kInfoThreads)
    if (p >= total) ids[p] = -1;
}

// ---------------------------------------------------------------------------
// event.csrmv kernels
// ---------------------------------------------------------------------------
template <typename IdxT>
__device__ __forceinline__ void row_bounds(const IdxT* indptr, int64_t row, int64_t nnz, int64_t& b, int64_t& e) {
  b = (int64_t)indptr[row];
  e = (int64_t)indptr[row + 1];
  b = b < 0 ? 0 : (b > nnz ? nnz : b);
  e = e < b ? b : (e > nnz ? nnz : e);
}

// transpose=1, one warp per active row, global atomics.
template <typename IdxT, bool HOMO>
__global__ void __launch_bounds__(256) ecsr_t_rowpar_kernel(const IdxT* __restrict__ indptr,
                                                            const IdxT* __restrict__ indices,
                                                            const float* __restrict__ data, int64_t nnz,
                                                            int64_t n, const int32_t* __restrict__ list,
                                                            const int32_t* __restrict__ count, void* out) {
  const int lane = lane_id();
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t a_total = *count;
  for (int64_t a = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); a < a_total; a += nwarps) {
    const int64_t row = list[a];
    int64_t b, e;
    row_bounds(indptr, row, nnz, b, e);
    int64_t j = b + lane;
    for (; j + 96 < e; j += 128) {
      int64_t c0 = (int64_t)indices[j], c1 = (int64_t)indices[j + 32];
      int64_t c2 = (int64_t)indices[j + 64], c3 = (int64_t)indices[j + 96];
      if (HOMO) {
        unsigned* o = static_cast<unsigned*>(out);
        if ((uint64_t)c0 < (uint64_t)n) atomicAdd(o + c0, 1u);
        if ((uint64_t)c1 < (uint64_t)n) atomicAdd(o + c1, 1u);
        if ((uint64_t)c2 < (uint64_t)n) atomicAdd(o + c2, 1u);
        if ((uint64_t)c3 < (uint64_t)n) atomicAdd(o + c3, 1u);
      } else {
        float w0 = data[j], w1 = data[j + 32], w2 = data[j + 64], w3 = data[j + 96];
        float* o = static_cast<float*>(out);
        if ((uint64_t)c0 < (uint64_t)n) atomicAdd(o + c0, w0);
        if ((uint64_t)c1 < (uint64_t)n) atomicAdd(o + c1, w1);
        if ((uint64_t)c2 < (uint64_t)n) atomicAdd(o + c2, w2);
        if ((uint64_t)c3 < (uint64_t)n) atomicAdd(o + c3, w3);
      }
    }
    for (; j < e; j += 32) {
      int64_t c = (int64_t)indices[j];
      if ((uint64_t)c < (uint64_t)n) {
        if (HOMO) atomicAdd(static_cast<unsigned*>(out) + c, 1u);
        else atomicAdd(static_cast<float*>(out) + c, data[j]);
      }
    }
  }
}

// counts (uint32, in place) -> float32 count * w
__global__ void counts_to_float_kernel(void* buf, int64_t n, const float* __restrict__ w_ptr) {
  const float w = *w_ptr;
  unsigned* u = static_cast<unsigned*>(buf);
  float* f = static_cast<float*>(buf);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    f[i] = (float)u[i] * w;
}

template <int ET>
__device__ __forceinline__ bool event_at(const void* events, int64_t i) {
  if (ET == BP_EV_BOOL) return __ldg(static_cast<const uint8_t*>(events) + i) != 0;
  return ev_on_f32(__ldg(static_cast<const float*>(events) + i), ET);
}

// transpose=1 on a small matrix, in one launch: a single CTA keeps the n output columns as
// shared-memory accumulators, compacts a round of events into a shared row list, scatters
// the listed rows (one warp per row, up to 128 entries per load round) and finally writes
// count * w (or the float sums) once.  No global atomics, no memsets, no second kernel:
// at the sizes of a 4000-neuron network the launches, not the bytes, are the cost of the
// general path.  Same arithmetic as the general path (exact uint32 counts for homogeneous
// weights, float32 sums otherwise).
constexpr int kSmallThreads = 1024;
constexpr int kSmallRound = kSmallThreads * 4;  // events examined per round (4 per thread)
constexpr int64_t kSmallMaxN = 49152;           // output words in shared memory (192 KB)
constexpr int64_t kSmallMaxM = 32768;           // at most 8 rounds of event scanning
constexpr int64_t kSmallMaxNnz = 1 << 19;       // worst case (every row active): 2^19 shared adds

static size_t small_smem_bytes(int64_t n) { return sizeof(uint32_t) * ((size_t)n + kSmallRound + 1); }

// Rows [r_begin, r_end) of a transposed product into the shared-memory accumulator `acc`
// (n words: u32 counts, or f32 sums): rounds of kSmallRound events compacted into the shared
// row list `rows`, then one warp per listed row, up to 128 entries a load round.
template <typename IdxT, bool HOMO, int ET>
__device__ __forceinline__ void small_scatter(uint32_t* acc, int32_t* rows, int32_t* n_rows, int64_t r_begin,
                                              int64_t r_end, const IdxT* __restrict__ indptr,
                                              const IdxT* __restrict__ indices, const float* __restrict__ data,
                                              int64_t nnz, int64_t n, const void* __restrict__ events) {
  const int lane = lane_id(), warp = threadIdx.x >> 5;
  constexpr int kWarps = kSmallThreads / 32;
  for (int64_t r0 = r_begin; r0 < r_end; r0 += kSmallRound) {
    if (threadIdx.x == 0) *n_rows = 0;
    __syncthreads();  // accumulators zeroed / previous round's list consumed
    bool on[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t r = r0 + u * kSmallThreads + threadIdx.x;
      on[u] = r < r_end && event_at<ET>(events, r);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const unsigned act = __ballot_sync(0xffffffffu, on[u]);
      if (!act) continue;
      int base = 0;
      if (lane == 0) base = atomicAdd(n_rows, __popc(act));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (on[u]) rows[base + __popc(act & ((1u << lane) - 1u))] = (int32_t)(r0 + u * kSmallThreads + threadIdx.x);
    }
    __syncthreads();
    const int cnt = *n_rows;
    for (int a = warp; a < cnt; a += kWarps) {
      int64_t b, e;
      row_bounds(indptr, (int64_t)rows[a], nnz, b, e);
      for (int64_t j0 = b; j0 < e; j0 += 128) {
        int64_t c[4];
        float w[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int64_t j = j0 + lane + 32 * u;
          c[u] = j < e ? (int64_t)indices[j] : -1;
          if (!HOMO) w[u] = j < e ? data[j] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if ((uint64_t)c[u] < (uint64_t)n) {
            if (HOMO) atomicAdd(acc + c[u], 1u);
            else atomicAdd(reinterpret_cast<float*>(acc) + c[u], w[u]);
          }
        }
      }
    }
    __syncthreads();  // the list is reused by the next round
  }
}

template <typename IdxT, bool HOMO, int ET>
__global__ void __launch_bounds__(kSmallThreads) ecsr_t_small_kernel(const IdxT* __restrict__ indptr,
                                                                     const IdxT* __restrict__ indices,
                                                                     const float* __restrict__ data, int64_t nnz,
                                                                     int64_t m, int64_t n,
                                                                     const void* __restrict__ events,
                                                                     float* __restrict__ out) {
  extern __shared__ uint32_t sm_small[];
  uint32_t* acc = sm_small;                                  // n words
  int32_t* rows = reinterpret_cast<int32_t*>(sm_small + n);  // kSmallRound row ids
  int32_t* n_rows = rows + kSmallRound;
  for (int64_t i = threadIdx.x; i < n; i += kSmallThreads) acc[i] = 0u;
  small_scatter<IdxT, HOMO, ET>(acc, rows, n_rows, 0, m, indptr, indices, data, nnz, n, events);
  __syncthreads();
  if (HOMO) {
    const float w0 = data[0];
    for (int64_t i = threadIdx.x; i < n; i += kSmallThreads) out[i] = (float)acc[i] * w0;
  } else {
    for (int64_t i = threadIdx.x; i < n; i += kSmallThreads) out[i] = __uint_as_float(acc[i]);
  }
}

// The same with one thread-block cluster of C CTAs, for small outputs with more work than one
// SM does quickly: every CTA holds all n columns, takes 1/C of the rows (scanning their events
// itself), and after a cluster barrier sums column slice q of the C accumulators through
// distributed shared memory (in rank order) and writes it.  Still one launch, no global
// atomics, no memset.
template <typename IdxT, bool HOMO, int ET>
__global__ void __launch_bounds__(kSmallThreads, 1) ecsr_t_cluster_small_kernel(const IdxT* __restrict__ indptr,
                                                                                const IdxT* __restrict__ indices,
                                                                                const float* __restrict__ data,
                                                                                int64_t nnz, int64_t m, int64_t n,
                                                                                const void* __restrict__ events,
                                                                                float* __restrict__ out) {
  extern __shared__ uint32_t sm_small[];
  uint32_t* acc = sm_small;
  int32_t* rows = reinterpret_cast<int32_t*>(sm_small + n);
  int32_t* n_rows = rows + kSmallRound;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks(), q = (int)cluster.block_rank();
  for (int64_t i = threadIdx.x; i < n; i += kSmallThreads) acc[i] = 0u;
  small_scatter<IdxT, HOMO, ET>(acc, rows, n_rows, q * m / C, (q + 1) * m / C, indptr, indices, data, nnz, n,
                                events);
  cluster.sync();  // every CTA's accumulator is complete
  const int64_t c0 = q * n / C, c1 = (q + 1) * n / C;
  const float w0 = HOMO ? data[0] : 0.0f;
  for (int64_t i = c0 + threadIdx.x; i < c1; i += kSmallThreads) {
    if (HOMO) {
      uint32_t s = 0;
      for (int r = 0; r < C; ++r) s += cluster.map_shared_rank(acc, r)[i];
      out[i] = (float)s * w0;
    } else {
      float s = 0.0f;
      for (int r = 0; r < C; ++r) s += __uint_as_float(cluster.map_shared_rank(acc, r)[i]);
      out[i] = s;
    }
  }
  cluster.sync();  // no CTA leaves while another may still read its accumulator
}

// transpose=0, one warp per row.
template <typename IdxT, bool HOMO, int ET>
__global__ void __launch_bounds__(256) ecsr_n_kernel(const IdxT* __restrict__ indptr,
                                                     const IdxT* __restrict__ indices,
                                                     const float* __restrict__ data, int64_t nnz, int64_t m,
                                                     int64_t n, const void* __restrict__ events,
                                                     float* __restrict__ out) {
  const int lane = lane_id();
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < m; row += nwarps) {
    int64_t b, e;
    row_bounds(indptr, row, nnz, b, e);
    unsigned cnt = 0;
    float acc = 0.0f;
    for (int64_t j = b + lane; j < e; j += 32) {
      int64_t c = (int64_t)indices[j];
      bool on = (uint64_t)c < (uint64_t)n && event_at<ET>(events, c);
      if (HOMO) cnt += on;
      else if (on) acc += data[j];
    }
    if (HOMO) {
      cnt = warp_sum(cnt);
      if (lane == 0) out[row] = (float)cnt * data[0];
    } else {
      acc = warp_sum(acc);
      if (lane == 0) out[row] = acc;
    }
  }
}

// transpose=0 when the event vector fits shared memory as bits (n <= kEvBitsMax * 8): one CTA
// per SM packs the events into bits once, then its warps stride over rows, each lane keeping
// kNBitsUnroll index loads in flight and testing the bits in shared memory -- no per-entry
// gather from L2.
// Same arithmetic as ecsr_n_kernel (counts, or the lane's in-order sum of weights).
constexpr size_t kEvBitsMax = 200 * 1024;
constexpr int kNBitsUnroll = 16;

template <typename IdxT, bool HOMO, int ET>
__global__ void __launch_bounds__(1024, 1) ecsr_n_bits_kernel(const IdxT* __restrict__ indptr,
                                                              const IdxT* __restrict__ indices,
                                                              const float* __restrict__ data, int64_t nnz, int64_t m,
                                                              int64_t n, const void* __restrict__ events,
                                                              float* __restrict__ out) {
  extern __shared__ uint32_t evb[];
  const bool vec_ok = ((reinterpret_cast<uintptr_t>(events) & 15u) == 0);
  const int64_t nw = (n + 31) / 32;
  for (int64_t w = threadIdx.x; w < nw; w += blockDim.x) {
    const int64_t base = w * 32;
    evb[w] = load_event_mask16<ET>(events, base, n, vec_ok) |
             (load_event_mask16<ET>(events, base + 16, n, vec_ok) << 16);
  }
  __syncthreads();
  const int lane = lane_id();
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < m; row += nwarps) {
    int64_t b, e;
    row_bounds(indptr, row, nnz, b, e);
    unsigned cnt = 0;
    float acc = 0.0f;
    for (int64_t j0 = b + lane; j0 < e; j0 += 32 * kNBitsUnroll) {
      int64_t c[kNBitsUnroll];
#pragma unroll
      for (int u = 0; u < kNBitsUnroll; ++u) c[u] = j0 + 32 * u < e ? (int64_t)indices[j0 + 32 * u] : -1;
#pragma unroll
      for (int u = 0; u < kNBitsUnroll; ++u) {
        const bool on = (uint64_t)c[u] < (uint64_t)n && ((evb[c[u] >> 5] >> (c[u] & 31)) & 1u);
        if (HOMO) cnt += on;
        else if (on) acc += data[j0 + 32 * u];
      }
    }
    if (HOMO) {
      cnt = warp_sum(cnt);
      if (lane == 0) out[row] = (float)cnt * data[0];
    } else {
      acc = warp_sum(acc);
      if (lane == 0) out[row] = acc;
    }
  }
}

template <typename IdxT, bool HOMO, int ET>
static bp_status launch_n_bits(const IdxT* indptr, const IdxT* indices, const float* data, int64_t nnz, int64_t m,
                               int64_t n, const void* events, float* out, cudaStream_t st) {
  auto kfn = ecsr_n_bits_kernel<IdxT, HOMO, ET>;
  static bool configured[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!configured[dev]) {
    BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kEvBitsMax));
    configured[dev] = true;
  }
  const size_t smem = (size_t)((n + 31) / 32) * sizeof(uint32_t);
  int64_t grid = (m + 31) / 32;
  if (grid > device_sm_count()) grid = device_sm_count();
  if (grid < 1) grid = 1;
  kfn<<<(unsigned)grid, 1024, smem, st>>>(indptr, indices, data, nnz, m, n, events, out);
  return check_launch("ecsr_n_bits_kernel");
}

static int grid_for(int64_t work_items, int per_block, int max_blocks) {
  int64_t g = (work_items + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (int)g;
}

template <int ET>
static bp_status launch_compact(const void* events, int64_t m, int32_t* list, int32_t* count, cudaStream_t st) {
  int grid = grid_for(m, 256 * 16, device_sm_count() * 8);
  compact_unordered_kernel<ET><<<grid, 256, 0, st>>>(events, m, list, count);
  return check_launch("compact_unordered_kernel");
}

bp_status compact_events(const void* events, bp_etype et, int64_t m, int32_t* list, int32_t* count,
                         cudaStream_t st) {
  switch (et) {
    case BP_EV_BOOL: return launch_compact<BP_EV_BOOL>(events, m, list, count, st);
    case BP_EV_F32_POS: return launch_compact<BP_EV_F32_POS>(events, m, list, count, st);
    case BP_EV_F32_NZ: return launch_compact<BP_EV_F32_NZ>(events, m, list, count, st);
  }
  return BP_EINVAL;
}

constexpr int64_t kClusterSmallMaxM = 1 << 18;    // rows scanned by the cluster's CTAs
constexpr int64_t kClusterSmallMaxNnz = 1 << 26;  // worst case: 2^22 shared adds per CTA at 16

// Largest cluster (16, else 8) of the small-output kernel that can be resident, 0 if none.
template <typename K>
static int small_cluster_size(K kfn, size_t smem) {
  for (int C : {16, 8}) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C, 1, 1);
    cfg.blockDim = dim3(kSmallThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kfn, &cfg) == cudaSuccess && clusters >= 1) return C;
    cudaGetLastError();
  }
  return 0;
}

template <typename IdxT, bool HOMO, int ET>
static bp_status launch_t_small(const IdxT* indptr, const IdxT* indices, const float* data, int64_t nnz, int64_t m,
                                int64_t n, const void* events, float* out, bool cluster, bool& done,
                                cudaStream_t st) {
  done = false;
  const size_t smem = small_smem_bytes(n);
  const size_t smem_max = small_smem_bytes(kSmallMaxN);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cluster) {
    auto kfn = ecsr_t_small_kernel<IdxT, HOMO, ET>;
    static bool configured[64] = {false};
    if (smem > 48 * 1024 && !configured[dev]) {
      BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
      configured[dev] = true;
    }
    {
      ScopedKernelTimer tk(st);
      kfn<<<1, kSmallThreads, smem, st>>>(indptr, indices, data, nnz, m, n, events, out);
    }
    done = true;
    return check_launch("ecsr_t_small_kernel");
  }
  auto kfn = ecsr_t_cluster_small_kernel<IdxT, HOMO, ET>;
  static int csize[64] = {0};  // 0: not probed yet, -1: no cluster resident
  if (csize[dev] == 0) {
    BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
    BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    const int c = small_cluster_size(kfn, smem_max);
    csize[dev] = c > 0 ? c : -1;
  }
  if (csize[dev] < 0) return BP_OK;  // not done: the caller takes the general path
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)csize[dev], 1, 1);
  cfg.blockDim = dim3(kSmallThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize[dev];
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  {
    ScopedKernelTimer tk(st);
    BP_CUDA_TRY(cudaLaunchKernelEx(&cfg, kfn, indptr, indices, data, nnz, m, n, events, out));
  }
  done = true;
  return check_launch("ecsr_t_cluster_small_kernel");
}

template <typename IdxT, bool HOMO>
static bp_status ecsr_t_small(const IdxT* indptr, const IdxT* indices, const float* data, int64_t nnz, int64_t m,
                              int64_t n, const void* events, bp_etype et, float* out, bool cluster, bool& done,
                              cudaStream_t st) {
  switch (et) {
    case BP_EV_BOOL:
      return launch_t_small<IdxT, HOMO, BP_EV_BOOL>(indptr, indices, data, nnz, m, n, events, out, cluster, done, st);
    case BP_EV_F32_POS:
      return launch_t_small<IdxT, HOMO, BP_EV_F32_POS>(indptr, indices, data, nnz, m, n, events, out, cluster, done,
                                                       st);
    case BP_EV_F32_NZ:
      return launch_t_small<IdxT, HOMO, BP_EV_F32_NZ>(indptr, indices, data, nnz, m, n, events, out, cluster, done,
                                                      st);
  }
  return BP_EINVAL;
}

// Whether a transposed product goes through the single-CTA kernel, or the one-cluster kernel.
static bool t_small_fits(int64_t m, int64_t n, int64_t nnz) {
  return m <= kSmallMaxM && n <= kSmallMaxN && nnz <= kSmallMaxNnz;
}
static bool t_cluster_small_fits(int64_t m, int64_t n, int64_t nnz) {
  return m <= kClusterSmallMaxM && n <= kSmallMaxN && nnz <= kClusterSmallMaxNnz;
}

template <typename IdxT>
static bp_status ecsr_transpose_rowpar(const float* data, bool homo, const IdxT* indices, const IdxT* indptr,
                                       int64_t nnz, const void* events, bp_etype et, int64_t m, int64_t n,
                                       float* out, int32_t* list, int32_t* count, cudaStream_t st) {
  const bool one = t_small_fits(m, n, nnz);
  if (one || t_cluster_small_fits(m, n, nnz)) {
    bool done = false;
    const bp_status s0 = homo ? ecsr_t_small<IdxT, true>(indptr, indices, data, nnz, m, n, events, et, out, !one, done, st)
                              : ecsr_t_small<IdxT, false>(indptr, indices, data, nnz, m, n, events, et, out, !one, done,
                                                          st);
    if (s0 != BP_OK || done) return s0;
  }
  BP_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(int32_t), st));
  BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n, st));
  bp_status s = compact_events(events, et, m, list, count, st);
  if (s != BP_OK) return s;
  const int grid = device_sm_count() * 8;
  {
    ScopedKernelTimer tk(st);
    if (homo) ecsr_t_rowpar_kernel<IdxT, true><<<grid, 256, 0, st>>>(indptr, indices, data, nnz, n, list, count, out);
    else ecsr_t_rowpar_kernel<IdxT, false><<<grid, 256, 0, st>>>(indptr, indices, data, nnz, n, list, count, out);
  }
  if ((s = check_launch("ecsr_t_rowpar_kernel")) != BP_OK) return s;
  if (homo) {
    counts_to_float_kernel<<<grid_for(n, 256 * 4, device_sm_count() * 8), 256, 0, st>>>(out, n, data);
    if ((s = check_launch("counts_to_float_kernel")) != BP_OK) return s;
  }
  return BP_OK;
}

// The transpose (event-driven) path on scratch supplied by the caller: `list` has room for
// m int32 row ids and `count` is one int32 (both are reset here before use).
bp_status event_csrmv_transpose_on_scratch(const float* data, bool homo, const void* indices, const void* indptr,
                                           bp_itype itype, int64_t nnz, const void* events, bp_etype et,
                                           int64_t m, int64_t n, float* out, int32_t* list, int32_t* count,
                                           cudaStream_t st) {
  if (itype == BP_I32)
    return ecsr_transpose_rowpar<int32_t>(data, homo, static_cast<const int32_t*>(indices),
                                          static_cast<const int32_t*>(indptr), nnz, events, et, m, n, out, list,
                                          count, st);
  return ecsr_transpose_rowpar<int64_t>(data, homo, static_cast<const int64_t*>(indices),
                                        static_cast<const int64_t*>(indptr), nnz, events, et, m, n, out, list,
                                        count, st);
}

template <typename IdxT, bool HOMO>
static bp_status ecsr_n_dispatch(const float* data, const IdxT* indices, const IdxT* indptr, int64_t nnz,
                                 const void* events, bp_etype et, int64_t m, int64_t n, float* out,
                                 cudaStream_t st) {
  ScopedKernelTimer tk(st);
  if ((size_t)((n + 31) / 32) * sizeof(uint32_t) <= kEvBitsMax && m >= 4096) {
    switch (et) {
      case BP_EV_BOOL: return launch_n_bits<IdxT, HOMO, BP_EV_BOOL>(indptr, indices, data, nnz, m, n, events, out, st);
      case BP_EV_F32_POS:
        return launch_n_bits<IdxT, HOMO, BP_EV_F32_POS>(indptr, indices, data, nnz, m, n, events, out, st);
      case BP_EV_F32_NZ:
        return launch_n_bits<IdxT, HOMO, BP_EV_F32_NZ>(indptr, indices, data, nnz, m, n, events, out, st);
    }
  }
  const int grid = grid_for(m, 8, device_sm_count() * 16);
  switch (et) {
    case BP_EV_BOOL:
      ecsr_n_kernel<IdxT, HOMO, BP_EV_BOOL><<<grid, 256, 0, st>>>(indptr, indices, data, nnz, m, n, events, out);
      break;
    case BP_EV_F32_POS:
      ecsr_n_kernel<IdxT, HOMO, BP_EV_F32_POS><<<grid, 256, 0, st>>>(indptr, indices, data, nnz, m, n, events, out);
      break;
    case BP_EV_F32_NZ:
      ecsr_n_kernel<IdxT, HOMO, BP_EV_F32_NZ><<<grid, 256, 0, st>>>(indptr, indices, data, nnz, m, n, events, out);
      break;
  }
  return check_launch("ecsr_n_kernel");
}

}  // namespace bp

using namespace bp;

extern "C" {

size_t bp_event_info_workspace_size(int64_t n) {
  int64_t nb = (n + kInfoChunk - 1) / kInfoChunk;
  return align_up(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1), 256);
}

bp_status bp_event_info(const void* events, bp_etype etype, int64_t n, int32_t* ids, int32_t* num_out,
                        void* workspace, size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(n >= 0, BP_EINVAL, "event_info: negative size %lld", (long long)n);
  BP_REQUIRE(n <= INT32_MAX, BP_ENOTSUP, "event_info: n=%lld exceeds int32 ids", (long long)n);
  BP_REQUIRE(etype >= BP_EV_BOOL && etype <= BP_EV_F32_NZ, BP_EINVAL, "event_info: bad etype %d", (int)etype);
  BP_REQUIRE(num_out != nullptr, BP_EINVAL, "event_info: num_out is null");
  if (n == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(num_out, 0, sizeof(int32_t), st));
    return BP_OK;
  }
  BP_REQUIRE(events && ids, BP_EINVAL, "event_info: null events/ids");
  BP_REQUIRE(workspace_bytes >= bp_event_info_workspace_size(n) && workspace, BP_ENOMEM,
             "event_info: workspace %zu < %zu", workspace_bytes, bp_event_info_workspace_size(n));
  int nb = (int)((n + kInfoChunk - 1) / kInfoChunk);
  int32_t* bc = static_cast<int32_t*>(workspace);
  switch (etype) {
    case BP_EV_BOOL: info_count_kernel<BP_EV_BOOL><<<nb, kInfoThreads, 0, st>>>(events, n, bc); break;
    case BP_EV_F32_POS: info_count_kernel<BP_EV_F32_POS><<<nb, kInfoThreads, 0, st>>>(events, n, bc); break;
    case BP_EV_F32_NZ: info_count_kernel<BP_EV_F32_NZ><<<nb, kInfoThreads, 0, st>>>(events, n, bc); break;
  }
  bp_status s = check_launch("info_count_kernel");
  if (s != BP_OK) return s;
  info_scan_kernel<<<1, 1024, 0, st>>>(bc, nb, num_out);
  if ((s = check_launch("info_scan_kernel")) != BP_OK) return s;
  switch (etype) {
    case BP_EV_BOOL: info_write_kernel<BP_EV_BOOL><<<nb, kInfoThreads, 0, st>>>(events, n, bc, num_out, ids); break;
    case BP_EV_F32_POS: info_write_kernel<BP_EV_F32_POS><<<nb, kInfoThreads, 0, st>>>(events, n, bc, num_out, ids); break;
    case BP_EV_F32_NZ: info_write_kernel<BP_EV_F32_NZ><<<nb, kInfoThreads, 0, st>>>(events, n, bc, num_out, ids); break;
  }
  return check_launch("info_write_kernel");
}

size_t bp_event_csrmv_workspace_size(int64_t m, int64_t n, int32_t transpose) {
  (void)n;
  if (!transpose) return 0;
  return 256 + align_up(sizeof(int32_t) * (size_t)(m > 0 ? m : 1), 256);
}

bp_status bp_event_csrmv(const float* data, int64_t ndata, const void* indices, const void* indptr,
                         bp_itype itype, int64_t nnz, const void* events, bp_etype etype, int64_t m,
                         int64_t n, int32_t transpose, float* out, void* workspace,
                         size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(m >= 0 && n >= 0 && nnz >= 0, BP_EINVAL, "event_csrmv: negative size m=%lld n=%lld nnz=%lld",
             (long long)m, (long long)n, (long long)nnz);
  BP_REQUIRE(m <= INT32_MAX && n <= INT32_MAX, BP_ENOTSUP, "event_csrmv: dimensions beyond int32 range");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "event_csrmv: bad index type %d", (int)itype);
  BP_REQUIRE(etype >= BP_EV_BOOL && etype <= BP_EV_F32_NZ, BP_EDTYPE, "event_csrmv: bad event type %d", (int)etype);
  BP_REQUIRE(ndata == 1 || ndata == nnz, BP_ESHAPE,
             "event_csrmv: the size of data should be 1 or be consistent with indices (%lld vs %lld)",
             (long long)ndata, (long long)nnz);
  const int64_t n_out = transpose ? n : m;
  if (n_out == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "event_csrmv: null out");
  if (m == 0 || nnz == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n_out, st));
    return BP_OK;
  }
  BP_REQUIRE(data && indices && indptr && events, BP_EINVAL, "event_csrmv: null data/indices/indptr/events");
  const bool homo = ndata == 1;
  if (transpose) {
    BP_REQUIRE(workspace && workspace_bytes >= bp_event_csrmv_workspace_size(m, n, 1), BP_ENOMEM,
               "event_csrmv: workspace %zu < %zu", workspace_bytes, bp_event_csrmv_workspace_size(m, n, 1));
    int32_t* count = static_cast<int32_t*>(workspace);
    int32_t* list = reinterpret_cast<int32_t*>(static_cast<char*>(workspace) + 256);
    if (itype == BP_I32)
      return ecsr_transpose_rowpar<int32_t>(data, homo, static_cast<const int32_t*>(indices),
                                            static_cast<const int32_t*>(indptr), nnz, events, etype, m, n, out,
                                            list, count, st);
    return ecsr_transpose_rowpar<int64_t>(data, homo, static_cast<const int64_t*>(indices),
                                          static_cast<const int64_t*>(indptr), nnz, events, etype, m, n, out, list,
                                          count, st);
  }
  if (itype == BP_I32) {
    auto ix = static_cast<const int32_t*>(indices);
    auto ip = static_cast<const int32_t*>(indptr);
    return homo ? ecsr_n_dispatch<int32_t, true>(data, ix, ip, nnz, events, etype, m, n, out, st)
                : ecsr_n_dispatch<int32_t, false>(data, ix, ip, nnz, events, etype, m, n, out, st);
  }
  auto ix = static_cast<const int64_t*>(indices);
  auto ip = static_cast<const int64_t*>(indptr);
  return homo ? ecsr_n_dispatch<int64_t, true>(data, ix, ip, nnz, events, etype, m, n, out, st)
              : ecsr_n_dispatch<int64_t, false>(data, ix, ip, nnz, events, etype, m, n, out, st);
}

}  // extern "C"
