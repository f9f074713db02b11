// net.cu -- LIF/Expon/COBA neuron update and whole-network persistent simulation.
//
// bp_lif_coba_step: one thread per neuron, the per-operator building block.
//
// bp_net_run: E/I COBA networks of up to 16 x 4096 neurons, each simulated by one thread-block
// cluster for many steps inside a single launch.  CTA `rank` owns neurons
// [rank*tile_w, (rank+1)*tile_w): their state, their two conductance event counters and the
// list of their spikes live in shared memory.  Step s:
//   1. propagation of step s-1's spikes: every CTA reads all ranks' spike lists through
//      distributed shared memory and, for each spiking row, streams that row's plan segment for
//      its own tile (tile-local uint16 indices), counting events per post-synaptic neuron with
//      shared-memory atomics, separately for excitatory and inhibitory rows;
//   2. neuron update with dge = count_e * we, dgi = count_i * wi; new spikes go into the other
//      half of a double-buffered list;
//   3. one cluster barrier.
// Reference order of a step (align_post.py:271-275, lif.py:461-500): the projections add the
// previous step's spike currents to the conductances, then the neurons update.
#include <cooperative_groups.h>

#include "common.cuh"
#include "lif.cuh"
#include "timer.cuh"

namespace cg = cooperative_groups;

namespace bp {

constexpr int kNetTileW = 4096;
constexpr int kNetMaxTiles = 16;
constexpr int kNetMaxDelay = 64;  // delay steps a network may hold (spike-history slots)
constexpr int kNetThreads = 1024;

__global__ void __launch_bounds__(256) lif_step_kernel(bp_lif_params p, int64_t n, float* __restrict__ V,
                                                       float* __restrict__ ge, float* __restrict__ gi,
                                                       float* __restrict__ t_last, uint8_t* __restrict__ spike,
                                                       const float* __restrict__ dge, const float* __restrict__ dgi,
                                                       int32_t step, const int32_t* __restrict__ step_dev, float dt) {
  const int32_t i = step_dev ? __ldg(step_dev) + step : step;
  const float t = __fmul_rn((float)i, dt);
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    LifState s{V[k], ge[k], gi[k], t_last[k]};
    const bool sp = lif_coba_update(p, s, dge ? dge[k] : 0.0f, dgi ? dgi[k] : 0.0f, t, dt);
    V[k] = s.V;
    ge[k] = s.ge;
    gi[k] = s.gi;
    t_last[k] = s.t_last;
    spike[k] = sp ? 1 : 0;
  }
}

struct NetSmem {
  float V[kNetTileW], ge[kNetTileW], gi[kNetTileW], tl[kNetTileW];
  uint32_t acc_e[kNetTileW], acc_i[kNetTileW];
  int32_t list[2][kNetTileW];
  int32_t cnt[2];
  int32_t nnew;                                 // spikes of the step being computed
  uint32_t ring[kNetMaxDelay][kNetTileW / 32];  // spike bits of the last L steps (step T in slot T mod L)
};

__device__ __forceinline__ int net_pos_mod(int64_t a, int L) { return (int)(((a % L) + L) % L); }

// bits of word w (32 neurons from base + 32 w) that are excitatory (global index < n_exc)
__device__ __forceinline__ uint32_t exc_bits(int base, int w, int n_exc) {
  const int lo = base + 32 * w;
  if (lo + 32 <= n_exc) return 0xffffffffu;
  if (lo >= n_exc) return 0u;
  return (1u << (n_exc - lo)) - 1u;
}

__global__ void __launch_bounds__(kNetThreads, 1) net_cluster_kernel(const bp_net_desc* __restrict__ descs,
                                                                     int32_t step0, int32_t steps, float dt) {
  extern __shared__ uint4 smem_raw[];
  NetSmem& S = *reinterpret_cast<NetSmem*>(smem_raw);
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const bp_net_desc d = descs[blockIdx.x / C];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int tw = d.tile_w;
  const int base = rank * tw;
  const int nloc = max(0, min(tw, d.n - base));
  const int words = (d.n + 31) >> 5;
  const int64_t toff_stride = d.n_tiles + 1;

  // Synaptic delays (VarDelay, brainpy/_src/delay.py:334-373): the excitatory rows propagate the
  // spikes of step T - d_e, the inhibitory rows those of T - d_i (d = 0 means the previous
  // step's spikes, the neurons' current spike state).  Spike bits of the last L steps live in
  // S.ring (step T in slot T mod L), loaded from and stored back to d.ring ([L][ceil(n/32)]).
  const int L = (d.ring != nullptr && d.ring_len > 0) ? min((int)d.ring_len, kNetMaxDelay) : 0;
  const int d_e = L ? max(0, min((int)d.delay_e, L)) : 0;
  const int d_i = L ? max(0, min((int)d.delay_i, L)) : 0;
  const int eff_e = max(d_e, 1), eff_i = max(d_i, 1);
  const int words_tile = tw >> 5, word0 = base >> 5;
  const int64_t T0 = (int64_t)step0 + d.step0;  // time index of this launch's first step
  // every word of the L slots is set (words past the tile to zero): the warps of the last
  // 1024-neuron round of a tile narrower than a multiple of 1024 read them
  for (int q = 0; q < L; ++q)
    for (int w = tid; w < kNetTileW / 32; w += blockDim.x)
      S.ring[q][w] = (w < words_tile && word0 + w < words) ? d.ring[(int64_t)q * words + word0 + w] : 0u;

  // load state, zero counters, initial spike list
  if (tid < 2) S.cnt[tid] = 0;
  for (int k = tid; k < tw; k += blockDim.x) {
    const bool in = k < nloc;
    S.V[k] = in ? d.V[base + k] : 0.0f;
    S.ge[k] = in ? d.ge[base + k] : 0.0f;
    S.gi[k] = in ? d.gi[base + k] : 0.0f;
    S.tl[k] = in ? d.t_last[base + k] : 0.0f;
    S.acc_e[k] = 0u;
    S.acc_i[k] = 0u;
  }
  __syncthreads();
  for (int k0 = 0; k0 < tw; k0 += blockDim.x) {
    const int k = k0 + tid;
    unsigned m = __ballot_sync(0xffffffffu, k < nloc && d.spike[base + k]);
    if (L) {  // the rows' delayed spikes for step T0, restricted to this tile's neurons
      const uint32_t em = exc_bits(base, k >> 5, d.n_exc);
      const uint32_t me = d_e == 0 ? m : S.ring[net_pos_mod(T0 - d_e, L)][k >> 5];
      const uint32_t mi = d_i == 0 ? m : S.ring[net_pos_mod(T0 - d_i, L)][k >> 5];
      m = ((me & em) | (mi & ~em)) & __ballot_sync(0xffffffffu, k < nloc);
    }
    const bool sp = (m >> lane) & 1u;
    int pos = 0;
    if (lane == 0 && m) pos = atomicAdd(&S.cnt[0], __popc(m));
    pos = __shfl_sync(0xffffffffu, pos, 0);
    if (sp) S.list[0][pos + __popc(m & ((1u << lane) - 1u))] = k;
  }
  cluster.sync();

  const int my_steps = d.step_limit > 0 ? min(steps, d.step_limit) : steps;
  // history slots of step T (written) and of T + 1 - eff_e / eff_i (read for the next step's
  // list), advanced by one each step (no division in the loop)
  int slot_w = 0, slot_e = 0, slot_i = 0;
  if (L) {
    slot_w = net_pos_mod(T0, L);
    slot_e = net_pos_mod(T0 + 1 - eff_e, L);
    slot_i = net_pos_mod(T0 + 1 - eff_i, L);
  }
  for (int s = 0; s < my_steps; ++s) {
    const int cur = s & 1, nxt = cur ^ 1;
    // ---- 1. propagate the previous step's spikes into this tile's counters
    int pre[kNetMaxTiles + 1];
    pre[0] = 0;
    for (int r = 0; r < C; ++r) pre[r + 1] = pre[r] + *cluster.map_shared_rank(&S.cnt[cur], r);
    const int total = pre[C];
    for (int g0 = warp * 32; g0 < total; g0 += nwarps * 32) {
      const int g = g0 + lane;
      uint32_t st = 0, nch = 0;
      bool exc = false;
      if (g < total) {
        int r = 0;
        while (pre[r + 1] <= g) ++r;
        const int32_t kloc = *cluster.map_shared_rank(&S.list[cur][g - pre[r]], r);
        const int64_t row = (int64_t)r * tw + kloc;
        exc = row < d.n_exc;
        const uint32_t* so = d.seg_off + row * toff_stride + rank;
        st = __ldg(so);
        nch = __ldg(so + 1) - st;
      }
      uint32_t* acc = exc ? S.acc_e : S.acc_i;
      constexpr int U = 4;
      for (uint32_t c0 = 0; __any_sync(0xffffffffu, c0 < nch); c0 += U) {
        uint4 vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (c0 + u < nch) vv[u] = __ldg(reinterpret_cast<const uint4*>(d.idx + 8ull * (st + c0 + u)));
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (c0 + u < nch) {
            const uint32_t x[8] = {vv[u].x & 0xFFFFu, vv[u].x >> 16, vv[u].y & 0xFFFFu, vv[u].y >> 16,
                                   vv[u].z & 0xFFFFu, vv[u].z >> 16, vv[u].w & 0xFFFFu, vv[u].w >> 16};
#pragma unroll
            for (int q = 0; q < 8; ++q)
              if (x[q] < (uint32_t)nloc) atomicAdd(acc + x[q], 1u);
          }
        }
      }
    }
    __syncthreads();
    // ---- 2. neuron update
    const float t = __fmul_rn((float)(step0 + d.step0 + s), dt);
    if (tid == 0) {
      S.cnt[nxt] = 0;
      S.nnew = 0;
    }
    __syncthreads();
    for (int k0 = 0; k0 < tw; k0 += blockDim.x) {
      const int k = k0 + tid;
      bool sp = false;
      if (k < nloc) {
        LifState st{S.V[k], S.ge[k], S.gi[k], S.tl[k]};
        const float dge = __fmul_rn((float)S.acc_e[k], d.we);
        const float dgi = __fmul_rn((float)S.acc_i[k], d.wi);
        S.acc_e[k] = 0u;
        S.acc_i[k] = 0u;
        sp = lif_coba_update(d.p, st, dge, dgi, t, dt);
        S.V[k] = st.V;
        S.ge[k] = st.ge;
        S.gi[k] = st.gi;
        S.tl[k] = st.t_last;
        if (d.v_trace && s < d.trace_steps) d.v_trace[(int64_t)s * d.n + base + k] = st.V;
      }
      const unsigned m = __ballot_sync(0xffffffffu, sp);
      if (d.raster && lane == 0 && k - lane < nloc)
        d.raster[(int64_t)s * words + ((base + k - lane) >> 5)] = m;
      if (lane == 0 && m) atomicAdd(&S.nnew, __popc(m));
      // the list the next step propagates: these spikes, or delayed ones from the ring
      unsigned ml = m;
      if (L) {
        if (lane == 0) S.ring[slot_w][k >> 5] = m;
        const uint32_t em = exc_bits(base, k >> 5, d.n_exc);
        const uint32_t me = eff_e == 1 ? m : S.ring[slot_e][k >> 5];
        const uint32_t mi = eff_i == 1 ? m : S.ring[slot_i][k >> 5];
        ml = ((me & em) | (mi & ~em)) & __ballot_sync(0xffffffffu, k < nloc);
      }
      int pos = 0;
      if (lane == 0 && ml) pos = atomicAdd(&S.cnt[nxt], __popc(ml));
      pos = __shfl_sync(0xffffffffu, pos, 0);
      if ((ml >> lane) & 1u) S.list[nxt][pos + __popc(ml & ((1u << lane) - 1u))] = k;
    }
    __syncthreads();
    if (tid == 0 && d.spike_counts && S.nnew) atomicAdd(d.spike_counts + s, S.nnew);
    if (L) {
      slot_w = slot_w + 1 == L ? 0 : slot_w + 1;
      slot_e = slot_e + 1 == L ? 0 : slot_e + 1;
      slot_i = slot_i + 1 == L ? 0 : slot_i + 1;
    }
    cluster.sync();
  }

  // write back state and the last step's spikes
  const int last = my_steps & 1;
  for (int k = tid; k < nloc; k += blockDim.x) {
    d.V[base + k] = S.V[k];
    d.ge[base + k] = S.ge[k];
    d.gi[base + k] = S.gi[k];
    d.t_last[base + k] = S.tl[k];
    if (L) {
      if (my_steps > 0) d.spike[base + k] = (S.ring[net_pos_mod(T0 + my_steps - 1, L)][k >> 5] >> (k & 31)) & 1u;
    } else {
      d.spike[base + k] = 0;
    }
  }
  for (int q = 0; q < L; ++q)
    for (int w = tid; w < words_tile; w += blockDim.x)
      if (word0 + w < words) d.ring[(int64_t)q * words + word0 + w] = S.ring[q][w];
  __syncthreads();
  if (!L)
    for (int j = tid; j < S.cnt[last]; j += blockDim.x) d.spike[base + S.list[last][j]] = 1;
  cluster.sync();  // no CTA leaves while another may still read its lists
}

// Spike history of the per-operator path (the persistent runner keeps the same layout in shared
// memory): ring[slot][w], bit b = neuron 32 w + b, step T in slot T mod L.  The time index is
// step (+ *step_dev when given, for CUDA-graph replay).
__global__ void __launch_bounds__(256) spike_ring_record_kernel(const uint8_t* __restrict__ spike, int64_t n,
                                                                uint32_t* __restrict__ ring, int32_t L, int64_t words,
                                                                int64_t step, const int32_t* __restrict__ step_dev) {
  const int64_t T = step + (step_dev ? (int64_t)__ldg(step_dev) : 0);
  uint32_t* row = ring + (int64_t)net_pos_mod(T, L) * words;
  const int lane = threadIdx.x & 31;
  for (int64_t k0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll; k0 < words * 32;
       k0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = k0 + lane;
    const uint32_t m = __ballot_sync(0xffffffffu, k < n && spike[k]);
    if (lane == 0) row[k0 >> 5] = m;
  }
}

// out[k] = bit of neuron lo + k in the slot of step T - delay (k < count)
__global__ void __launch_bounds__(256) spike_ring_read_kernel(const uint32_t* __restrict__ ring, int32_t L,
                                                              int64_t words, int64_t lo, int64_t count, int32_t delay,
                                                              int64_t step, const int32_t* __restrict__ step_dev,
                                                              uint8_t* __restrict__ out) {
  const int64_t T = step + (step_dev ? (int64_t)__ldg(step_dev) : 0);
  const uint32_t* row = ring + (int64_t)net_pos_mod(T - delay, L) * words;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = lo + k;
    out[k] = (uint8_t)((__ldg(row + (g >> 5)) >> (g & 31)) & 1u);
  }
}

}  // namespace bp

using namespace bp;

extern "C" {

bp_status bp_lif_coba_step(const bp_lif_params* params, int64_t n, float* V, float* ge, float* gi, float* t_last,
                           uint8_t* spike, const float* dge, const float* dgi, int32_t step, float dt,
                           bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(params != nullptr, BP_EINVAL, "lif_coba_step: null params");
  BP_REQUIRE(n >= 0, BP_EINVAL, "lif_coba_step: negative size");
  if (n == 0) return BP_OK;
  BP_REQUIRE(V && ge && gi && t_last && spike, BP_EINVAL, "lif_coba_step: null state");
  int64_t g = (n + 255) / 256;
  const int64_t maxb = (int64_t)device_sm_count() * 16;
  if (g > maxb) g = maxb;
  ScopedKernelTimer tk(st);
  lif_step_kernel<<<(int)g, 256, 0, st>>>(*params, n, V, ge, gi, t_last, spike, dge, dgi, step, nullptr, dt);
  return check_launch("lif_step_kernel");
}

bp_status bp_lif_coba_step_dev(const bp_lif_params* params, int64_t n, float* V, float* ge, float* gi,
                               float* t_last, uint8_t* spike, const float* dge, const float* dgi,
                               const int32_t* step_dev, int32_t step_offset, float dt, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(params != nullptr && step_dev != nullptr, BP_EINVAL, "lif_coba_step_dev: null params/step");
  BP_REQUIRE(n >= 0, BP_EINVAL, "lif_coba_step_dev: negative size");
  if (n == 0) return BP_OK;
  BP_REQUIRE(V && ge && gi && t_last && spike, BP_EINVAL, "lif_coba_step_dev: null state");
  int64_t g = (n + 255) / 256;
  const int64_t maxb = (int64_t)device_sm_count() * 16;
  if (g > maxb) g = maxb;
  lif_step_kernel<<<(int)g, 256, 0, st>>>(*params, n, V, ge, gi, t_last, spike, dge, dgi, step_offset, step_dev, dt);
  return check_launch("lif_step_kernel");
}

bp_status bp_spike_ring_record(const uint8_t* spike, int64_t n, uint32_t* ring, int32_t ring_len, int64_t step,
                               const int32_t* step_dev, bp_stream_t stream) {
  clear_error();
  BP_REQUIRE(n >= 0 && ring_len >= 1, BP_EINVAL, "spike_ring_record: n >= 0 and ring_len >= 1 required");
  if (n == 0) return BP_OK;
  BP_REQUIRE(spike && ring, BP_EINVAL, "spike_ring_record: null pointer");
  const int64_t words = (n + 31) / 32;
  int64_t g = (words * 32 + 255) / 256;
  const int64_t maxb = (int64_t)device_sm_count() * 16;
  if (g > maxb) g = maxb;
  spike_ring_record_kernel<<<(int)g, 256, 0, as_cuda(stream)>>>(spike, n, ring, ring_len, words, step, step_dev);
  return check_launch("spike_ring_record_kernel");
}

bp_status bp_spike_ring_read(const uint32_t* ring, int32_t ring_len, int64_t n, int64_t lo, int64_t count,
                             int32_t delay, int64_t step, const int32_t* step_dev, uint8_t* out, bp_stream_t stream) {
  clear_error();
  BP_REQUIRE(ring_len >= 1 && n >= 0 && lo >= 0 && count >= 0 && lo + count <= n, BP_EINVAL,
             "spike_ring_read: bad range [%lld, %lld) of %lld", (long long)lo, (long long)(lo + count), (long long)n);
  if (count == 0) return BP_OK;
  BP_REQUIRE(ring && out, BP_EINVAL, "spike_ring_read: null pointer");
  int64_t g = (count + 255) / 256;
  const int64_t maxb = (int64_t)device_sm_count() * 16;
  if (g > maxb) g = maxb;
  spike_ring_read_kernel<<<(int)g, 256, 0, as_cuda(stream)>>>(ring, ring_len, (n + 31) / 32, lo, count, delay, step,
                                                               step_dev, out);
  return check_launch("spike_ring_read_kernel");
}

int32_t bp_net_max_tiles(void) { return kNetMaxTiles; }
int32_t bp_net_tile_width(void) { return kNetTileW; }

bp_status bp_net_run(const bp_net_desc* descs_device, int32_t num_nets, int32_t cluster, int32_t step0,
                     int32_t steps, float dt, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(num_nets >= 0 && steps >= 0, BP_EINVAL, "net_run: negative count");
  BP_REQUIRE(cluster >= 1 && cluster <= kNetMaxTiles, BP_EINVAL, "net_run: cluster %d outside [1, %d]", cluster,
             kNetMaxTiles);
  if (num_nets == 0 || steps == 0) return BP_OK;
  BP_REQUIRE(descs_device != nullptr, BP_EINVAL, "net_run: null descriptors");
  auto kfn = net_cluster_kernel;
  const size_t smem = sizeof(NetSmem);
  static int configured[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!configured[dev]) {
    BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    configured[dev] = 1;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(num_nets * cluster), 1, 1);
  cfg.blockDim = dim3(kNetThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  ScopedKernelTimer tk(st);
  BP_CUDA_TRY(cudaLaunchKernelEx(&cfg, kfn, descs_device, step0, steps, dt));
  return BP_OK;
}

}  // extern "C"
