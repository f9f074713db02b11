// net_grid.cu -- E/I COBA networks too large for one thread-block cluster, simulated for many
// steps inside one persistent launch over the whole GPU.
//
// The network's CSR plan is cut into column tiles of tile_w neurons; each tile is owned by a
// cluster of kGridR CTAs, and CTA q of the cluster owns neurons [q*tile_w/R, (q+1)*tile_w/R)
// of the tile (their state stays in global memory; only this CTA touches it).  Step s:
//   1. propagation of step s-1's spikes: the spiking rows of the whole network (one list per
//      CTA in global memory, written in step s-1) are split over the cluster's CTAs; each CTA
//      streams those rows' plan segments for its tile and adds into a shared-memory counter
//      per column, excitatory rows in the low 16 bits, inhibitory rows in the high 16 bits
//      (the host checks that no column has 65,536 or more incoming entries);
//   2. after a cluster barrier every CTA sums the R counters of its own columns through
//      distributed shared memory and updates its neurons with dge = count_e * we and
//      dgi = count_i * wi (the same float32 operations as the per-operator path and the
//      oracle), writing its spikes into its list for the next step;
//   3. a cluster barrier (the counters are read), zeroing, and a grid-wide barrier (every list
//      of this step is complete).
// The grid barrier is this kernel's own: an arrival counter and a generation word in global
// memory, with a bounded spin.  A CTA whose wait runs out records an error and its whole
// cluster leaves at the next step (the decision is shared through distributed shared memory so
// that no cluster barrier waits on a CTA that left); the other clusters then run out at their
// next grid barrier.  The launch asks for cooperative scheduling, so all CTAs are resident.
// Reference order of a step (align_post.py:271-275, lif.py:461-500): the projections add the
// previous step's spike currents to the conductances, then the neurons update.
#include <cooperative_groups.h>

#include "common.cuh"
#include "lfsr88.cuh"
#include "lif.cuh"
#include "plan.cuh"
#include "timer.cuh"

namespace cg = cooperative_groups;

namespace bp {

constexpr int kGridR = 4;            // CTAs per tile (a cluster)
constexpr int kGridThreads = 1024;
constexpr int kGridTileAlign = 128;  // tile widths are multiples of this (R * 32)
constexpr int kGridMaxCtas = 1024;   // one prefix element per thread
constexpr unsigned kGridSpinLimit = 1u << 22;  // ~0.3-1 s of 64 ns sleeps
constexpr int kGridUpd = 4;          // neurons a thread updates per round (jitconn runner)

struct GridArgs {
  uint32_t* bar;    // [0] arrivals, [1] generation
  int32_t* err;     // set when a grid-barrier wait ran out
  int32_t* cnt;     // [2][G] spikes listed by each CTA
  int32_t* list;    // [2][G][slice] global neuron ids
  int32_t slice;    // neurons per CTA
};

static size_t grid_smem_bytes(int tile_w) {
  return sizeof(uint32_t) * (size_t)(tile_w + kPlanPadSpan) + sizeof(int32_t) * (size_t)(kGridMaxCtas + 1);
}

constexpr int kGridMaxDelay = 64;  // spike-history slots (as the cluster runner)

__device__ __forceinline__ int grid_pos_mod(int64_t a, int L) { return (int)(((a % L) + L) % L); }

// bits of the 32 neurons from lo that are excitatory (global index < n_exc)
__device__ __forceinline__ uint32_t grid_exc_bits(int64_t lo, int n_exc) {
  if (lo + 32 <= n_exc) return 0xffffffffu;
  if (lo >= n_exc) return 0u;
  return (1u << (n_exc - lo)) - 1u;
}

// Bounded grid-wide barrier; returns false when the wait ran out.
__device__ bool grid_barrier(const GridArgs& g, uint32_t nblocks, int* s_flag) {
  __threadfence();  // this thread's list / count writes before the arrival
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = g.bar + 1;
    const uint32_t my_gen = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(g.bar, 1u) == nblocks - 1u) {
      atomicExch(g.bar, 0u);
      __threadfence();
      atomicAdd(g.bar + 1, 1u);
    } else {
      uint32_t it = 0;
      while (*gen == my_gen) {
        if (++it > kGridSpinLimit) {
          ok = 0;
          atomicExch(g.err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    *s_flag = ok;
  }
  __syncthreads();
  return *s_flag != 0;
}

__global__ void __launch_bounds__(kGridThreads, 1) net_grid_kernel(const bp_net_desc d, int32_t step0, int32_t steps,
                                                                   float dt, const GridArgs g) {
  constexpr unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_ok, s_flag, s_count, s_nnew, s_wsum[32];
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  const int tile = (int)blockIdx.x / kGridR;
  const uint32_t G = gridDim.x;
  const int tw = d.tile_w;
  const int slice = g.slice;
  const int acc_words = tw + kPlanPadSpan;
  uint32_t* acc = reinterpret_cast<uint32_t*>(smem);
  const uint32_t acc_s = (uint32_t)__cvta_generic_to_shared(acc);
  int* s_pre = reinterpret_cast<int*>(acc + acc_words);  // G + 1
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int64_t base = (int64_t)tile * tw + (int64_t)q * slice;  // first neuron of this CTA
  const int64_t rem = (int64_t)d.n - base;
  const int nown = (int)(rem < 0 ? 0 : (rem > slice ? slice : rem));
  const int64_t so_stride = d.n_tiles + 1;

  auto zero_acc = [&]() {
    uint4* a4 = reinterpret_cast<uint4*>(acc);
    for (int i = tid; i < (acc_words >> 2); i += blockDim.x) a4[i] = make_uint4(0u, 0u, 0u, 0u);
  };
  // appends this warp's flagged neurons (bit l of m: this CTA's neuron kw + l, kw the warp's
  // first) to list[par][blockIdx.x]
  auto append = [&](int par, unsigned m, int kw) {
    int pos = 0;
    if (lane == 0 && m) pos = atomicAdd(&s_count, __popc(m));
    pos = __shfl_sync(FULL, pos, 0);
    int32_t* my_list = g.list + ((int64_t)par * G + blockIdx.x) * slice;
    if ((m >> lane) & 1u) my_list[pos + __popc(m & ((1u << lane) - 1u))] = (int32_t)(base + kw + lane);
  };

  // Synaptic delays (VarDelay, brainpy/_src/delay.py:334-373): the excitatory rows propagate
  // the spikes of step T - d_e, the inhibitory rows those of T - d_i (0: the previous step's
  // spikes).  The spike bits of the last L steps stay in d.ring ([L][ceil(n/32)], step T in
  // slot T mod L); this CTA's neurons are whole words of it (slice and base are multiples of
  // 32), which only this CTA reads and writes.
  const int L = (d.ring != nullptr && d.ring_len > 0) ? min((int)d.ring_len, kGridMaxDelay) : 0;
  const int d_e = L ? max(0, min((int)d.delay_e, L)) : 0;
  const int d_i = L ? max(0, min((int)d.delay_i, L)) : 0;
  const int eff_e = max(d_e, 1), eff_i = max(d_i, 1);
  const int64_t words = ((int64_t)d.n + 31) >> 5;
  const int64_t word0 = base >> 5;
  const int64_t T0 = (int64_t)step0 + d.step0;  // time index of this launch's first step
  auto ring_word = [&](int slot, int k) -> uint32_t {  // word of neurons base + (k & ~31) ..
    const int64_t w = word0 + (k >> 5);
    return w < words ? __ldcg(d.ring + (int64_t)slot * words + w) : 0u;
  };

  zero_acc();
  // the initial list: this CTA's neurons whose (delayed) spike the first step propagates
  if (tid == 0) s_count = 0;
  __syncthreads();
  for (int k0 = 0; k0 < slice; k0 += blockDim.x) {
    const int k = k0 + tid;
    unsigned m = __ballot_sync(FULL, k < nown && d.spike[base + k] != 0);
    if (L) {
      const uint32_t em = grid_exc_bits(base + (k & ~31), d.n_exc);
      const uint32_t me = d_e == 0 ? m : ring_word(grid_pos_mod(T0 - d_e, L), k);
      const uint32_t mi = d_i == 0 ? m : ring_word(grid_pos_mod(T0 - d_i, L), k);
      m = ((me & em) | (mi & ~em)) & __ballot_sync(FULL, k < nown);
    }
    append(0, m, k0 + (tid & ~31));
  }
  __syncthreads();
  if (tid == 0) g.cnt[blockIdx.x] = s_count;
  bool ok = grid_barrier(g, G, &s_flag);

  const int my_steps = d.step_limit > 0 ? min(steps, d.step_limit) : steps;
  // history slots of step T (written) and of T + 1 - eff_e / eff_i (read for the next list)
  int slot_w = 0, slot_e = 0, slot_i = 0;
  if (L) {
    slot_w = grid_pos_mod(T0, L);
    slot_e = grid_pos_mod(T0 + 1 - eff_e, L);
    slot_i = grid_pos_mod(T0 + 1 - eff_i, L);
  }
  for (int s = 0; s < my_steps; ++s) {
    const int cur = s & 1, nxt = cur ^ 1;
    // leave together when any CTA of the cluster saw a grid-barrier wait run out
    if (tid == 0) s_ok = ok ? 1 : 0;
    cluster.sync();
    int all_ok = 1;
    for (int r = 0; r < kGridR; ++r) all_ok &= *cluster.map_shared_rank(&s_ok, r);
    cluster.sync();
    if (!all_ok) break;

    // ---- 1. the spiking rows of step s-1 (every CTA's list), this CTA's share
    {
      const int v = tid < (int)G ? __ldcg(g.cnt + (int64_t)cur * G + tid) : 0;
      int incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      if (warp == 0) {
        const int t = lane < nwarps ? s_wsum[lane] : 0;
        int ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int u = __shfl_up_sync(FULL, ti, o);
          if (lane >= o) ti += u;
        }
        s_wsum[lane] = ti - t;
      }
      __syncthreads();
      if (tid < (int)G) s_pre[tid] = s_wsum[warp] + incl - v;
      if (tid == (int)G - 1) s_pre[G] = s_wsum[warp] + incl;
      __syncthreads();
    }
    const int total = s_pre[G];
    const int lo = (int)((int64_t)q * total / kGridR), hi = (int)((int64_t)(q + 1) * total / kGridR);
    for (int p0 = lo + warp * 32; p0 < hi; p0 += nwarps * 32) {
      const int p = p0 + lane;
      uint32_t st = 0, nch = 0, inc = 0;
      if (p < hi) {
        int l = 0, h = (int)G;  // s_pre[l] <= p < s_pre[h]
        while (h - l > 1) {
          const int mid = (l + h) >> 1;
          if (s_pre[mid] <= p) l = mid;
          else h = mid;
        }
        const int64_t row = __ldcg(g.list + ((int64_t)cur * G + l) * slice + (p - s_pre[l]));
        const uint32_t* so = d.seg_off + row * so_stride + tile;
        st = __ldg(so);
        nch = __ldg(so + 1) - st;
        inc = row < d.n_exc ? 1u : 0x10000u;
      }
      constexpr int U = 4;
      for (uint32_t c0 = 0; __any_sync(FULL, c0 < nch); c0 += U) {
        uint4 vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (c0 + u < nch) vv[u] = __ldg(reinterpret_cast<const uint4*>(d.idx + 8ull * (st + c0 + u)));
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (c0 + u < nch) {
            const uint32_t x[8] = {vv[u].x & 0xFFFFu, vv[u].x >> 16, vv[u].y & 0xFFFFu, vv[u].y >> 16,
                                   vv[u].z & 0xFFFFu, vv[u].z >> 16, vv[u].w & 0xFFFFu, vv[u].w >> 16};
            // pad entries (index tile_w and up) land on the spare words past the tile
#pragma unroll
            for (int e = 0; e < 8; ++e) asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(acc_s + 4u * x[e]), "r"(inc));
          }
        }
      }
    }
    cluster.sync();  // every CTA's counters of the tile are complete

    // ---- 2. this CTA's neurons: sum the cluster's counters, update, list the spikes
    const float t = __fmul_rn((float)(step0 + d.step0 + s), dt);
    if (tid == 0) {
      s_count = 0;
      s_nnew = 0;
    }
    __syncthreads();
    for (int k0 = 0; k0 < slice; k0 += blockDim.x) {
      const int k = k0 + tid;
      bool sp = false;
      if (k < nown) {
        const int col = q * slice + k;
        uint32_t packed = 0;
#pragma unroll
        for (int r = 0; r < kGridR; ++r) packed += *cluster.map_shared_rank(acc + col, r);
        const int64_t i = base + k;
        LifState st{d.V[i], d.ge[i], d.gi[i], d.t_last[i]};
        const float dge = __fmul_rn((float)(packed & 0xFFFFu), d.we);
        const float dgi = __fmul_rn((float)(packed >> 16), d.wi);
        sp = lif_coba_update(d.p, st, dge, dgi, t, dt);
        d.V[i] = st.V;
        d.ge[i] = st.ge;
        d.gi[i] = st.gi;
        d.t_last[i] = st.t_last;
        d.spike[i] = sp ? 1 : 0;
        if (d.v_trace && s < d.trace_steps) d.v_trace[(int64_t)s * d.n + i] = st.V;
      }
      const unsigned m = __ballot_sync(FULL, sp);
      if (lane == 0 && m) atomicAdd(&s_nnew, __popc(m));
      unsigned ml = m;  // the rows the next step propagates
      if (L) {
        // only this CTA's words: a warp past the slice (k0 rounds up to whole blocks of
        // threads) would otherwise write over the next CTA's first words
        const int64_t w = word0 + (k >> 5);
        if (lane == 0 && (k & ~31) < slice && w < words) d.ring[(int64_t)slot_w * words + w] = m;
        const uint32_t em = grid_exc_bits(base + (k & ~31), d.n_exc);
        const uint32_t me = eff_e == 1 ? m : ring_word(slot_e, k);
        const uint32_t mi = eff_i == 1 ? m : ring_word(slot_i, k);
        ml = ((me & em) | (mi & ~em)) & __ballot_sync(FULL, k < nown);
      }
      append(nxt, ml, k0 + (tid & ~31));
    }
    __syncthreads();
    if (tid == 0) {
      g.cnt[(int64_t)nxt * G + blockIdx.x] = s_count;
      if (d.spike_counts && s_nnew) atomicAdd(d.spike_counts + s, s_nnew);
    }
    if (L) {
      slot_w = slot_w + 1 == L ? 0 : slot_w + 1;
      slot_e = slot_e + 1 == L ? 0 : slot_e + 1;
      slot_i = slot_i + 1 == L ? 0 : slot_i + 1;
    }
    cluster.sync();  // the cluster's reads of this CTA's counters are done
    zero_acc();
    ok = grid_barrier(g, G, &s_flag) && ok;
  }
}

// ---------------------------------------------------------------------------
// Just-in-time networks, push form (EventJitFPHomoLinear with atomic=True: outdim_parallel=False),
// in one persistent launch: one CTA per SM owns a contiguous slice of neurons.  Step s:
//   1. the spiking neurons of step s-1 (the CTAs' lists) are split over every warp of the grid;
//      a warp regenerates a neuron's connections of both projections leaving its group, its 32
//      lanes walking the 32 streams of the Taichi GPU push algorithm (the streams and the adds
//      of jc_push_gpu_kernel: a homogeneous weight added once per connection with a float
//      atomic into dge or dgi in global memory; equal addends, so the order of the adds does
//      not change the sums and the result equals the per-operator path bit for bit);
//   2. a grid barrier; every CTA reads and zeroes dge / dgi of its neurons and updates them,
//      listing its spikes;
//   3. a grid barrier.
// The barrier and its bounded waits are those of the CSR runner; no clusters here, so a CTA
// whose wait runs out records the error and leaves, and the others run out at their next
// barrier.
// ---------------------------------------------------------------------------
struct JitGridArgs {
  uint32_t* bar;
  int32_t* err;
  int32_t* cnt;    // [2][G]
  int32_t* list;   // [2][G][slice]
  float* dge;      // [n], zero between steps
  float* dgi;      // [n]
  int32_t slice;
  uint32_t seed[4];          // E->E, E->I, I->E, I->I
  uint32_t step_e, step_i;   // lane window of the projections onto E rows / onto I rows
  FastMod fm;
};

__device__ __forceinline__ void jit_push(const JitGridArgs& g, uint32_t col, uint32_t seed, uint32_t nrow,
                                         uint32_t step, float* out, float w, int lane) {
  const uint32_t i = col * 32u + (uint32_t)lane;
  uint32_t r = step * (uint32_t)lane - 1u;
  uint32_t end = r + step;
  if (nrow < end) end = nrow;
  Lfsr88 key = lfsr88_key(seed + i);
  r += lfsr88_inc(key, g.fm);
  while (r < end) {
    atomicAdd(out + r, w);
    r += lfsr88_inc(key, g.fm);
  }
}

__global__ void __launch_bounds__(kGridThreads, 1) net_grid_jit_kernel(const bp_net_desc d, int32_t step0,
                                                                       int32_t steps, float dt, const JitGridArgs g) {
  constexpr unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_flag, s_count, s_wsum[32];
  int* s_pre = reinterpret_cast<int*>(smem);  // G + 1
  const uint32_t G = gridDim.x;
  const int slice = g.slice;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * slice;
  const int64_t rem = (int64_t)d.n - base;
  const int nown = (int)(rem < 0 ? 0 : (rem > slice ? slice : rem));
  const uint32_t ne = (uint32_t)d.n_exc, ni = (uint32_t)(d.n - d.n_exc);
  GridArgs gb;  // the barrier words of the CSR runner's layout
  gb.bar = g.bar;
  gb.err = g.err;

  auto append = [&](int par, unsigned m, int kw) {
    int pos = 0;
    if (lane == 0 && m) pos = atomicAdd(&s_count, __popc(m));
    pos = __shfl_sync(FULL, pos, 0);
    int32_t* my_list = g.list + ((int64_t)par * G + blockIdx.x) * slice;
    if ((m >> lane) & 1u) my_list[pos + __popc(m & ((1u << lane) - 1u))] = (int32_t)(base + kw + lane);
  };

  if (tid == 0) s_count = 0;
  __syncthreads();
  for (int k0 = 0; k0 < slice; k0 += blockDim.x) {
    const int k = k0 + tid;
    const unsigned m = __ballot_sync(FULL, k < nown && d.spike[base + k] != 0);
    append(0, m, k0 + (tid & ~31));
  }
  __syncthreads();
  if (tid == 0) g.cnt[blockIdx.x] = s_count;
  if (!grid_barrier(gb, G, &s_flag)) return;

  const int my_steps = d.step_limit > 0 ? min(steps, d.step_limit) : steps;
  for (int s = 0; s < my_steps; ++s) {
    const int cur = s & 1, nxt = cur ^ 1;
    // ---- 1. every spiking neuron of step s-1, this CTA's share, pushed by its warps
    {
      const int v = tid < (int)G ? __ldcg(g.cnt + (int64_t)cur * G + tid) : 0;
      int incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      if (warp == 0) {
        const int t = lane < nwarps ? s_wsum[lane] : 0;
        int ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int u = __shfl_up_sync(FULL, ti, o);
          if (lane >= o) ti += u;
        }
        s_wsum[lane] = ti - t;
      }
      __syncthreads();
      if (tid < (int)G) s_pre[tid] = s_wsum[warp] + incl - v;
      if (tid == (int)G - 1) s_pre[G] = s_wsum[warp] + incl;
      __syncthreads();
    }
    const int total = s_pre[G];
    const int lo = (int)((int64_t)blockIdx.x * total / G), hi = (int)((int64_t)(blockIdx.x + 1) * total / G);
    for (int p = lo + warp; p < hi; p += nwarps) {
      int l = 0, h = (int)G;  // s_pre[l] <= p < s_pre[h]
      while (h - l > 1) {
        const int mid = (l + h) >> 1;
        if (s_pre[mid] <= p) l = mid;
        else h = mid;
      }
      const uint32_t j = (uint32_t)__ldcg(g.list + ((int64_t)cur * G + l) * slice + (p - s_pre[l]));
      if (j < ne) {
        jit_push(g, j, g.seed[0], ne, g.step_e, g.dge, d.we, lane);
        jit_push(g, j, g.seed[1], ni, g.step_i, g.dge + ne, d.we, lane);
      } else {
        jit_push(g, j - ne, g.seed[2], ne, g.step_e, g.dgi, d.wi, lane);
        jit_push(g, j - ne, g.seed[3], ni, g.step_i, g.dgi + ne, d.wi, lane);
      }
    }
    if (!grid_barrier(gb, G, &s_flag)) return;  // every push of the step is in dge / dgi

    // ---- 2. this CTA's neurons
    const float t = __fmul_rn((float)(step0 + d.step0 + s), dt);
    if (tid == 0) s_count = 0;
    __syncthreads();
    // kGridUpd neurons a thread per round, their loads issued before any update
    for (int k00 = 0; k00 < slice; k00 += kGridUpd * kGridThreads) {
      LifState st[kGridUpd];
      float xe[kGridUpd], xi[kGridUpd];
#pragma unroll
      for (int u = 0; u < kGridUpd; ++u) {
        const int k = k00 + u * kGridThreads + tid;
        xe[u] = xi[u] = 0.0f;
        if (k < nown) {
          const int64_t i = base + k;
          xe[u] = __ldcg(g.dge + i);
          xi[u] = __ldcg(g.dgi + i);
          st[u] = LifState{d.V[i], d.ge[i], d.gi[i], d.t_last[i]};
        }
      }
#pragma unroll
      for (int u = 0; u < kGridUpd; ++u) {
        const int k0 = k00 + u * kGridThreads;
        const int k = k0 + tid;
        bool sp = false;
        if (k < nown) {
          const int64_t i = base + k;
          g.dge[i] = 0.0f;
          g.dgi[i] = 0.0f;
          sp = lif_coba_update(d.p, st[u], xe[u], xi[u], t, dt);
          d.V[i] = st[u].V;
          d.ge[i] = st[u].ge;
          d.gi[i] = st[u].gi;
          d.t_last[i] = st[u].t_last;
          d.spike[i] = sp ? 1 : 0;
          if (d.v_trace && s < d.trace_steps) d.v_trace[(int64_t)s * d.n + i] = st[u].V;
        }
        const unsigned m = __ballot_sync(FULL, sp);
        append(nxt, m, k0 + (tid & ~31));
      }
    }
    __syncthreads();
    if (tid == 0) {
      g.cnt[(int64_t)nxt * G + blockIdx.x] = s_count;
      if (d.spike_counts && s_count) atomicAdd(d.spike_counts + s, s_count);
    }
    if (!grid_barrier(gb, G, &s_flag)) return;
  }
}

static int grid_smem_optin() {
  static int cache[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (cache[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cache[dev] = v > 0 ? v : 227 * 1024;
  }
  return cache[dev];
}

static int grid_max_clusters(int tile_w) {
  static int cached[64][2] = {};  // [device] -> {tile_w, clusters}
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (cached[dev][0] == tile_w && cached[dev][1] > 0) return cached[dev][1];
  const size_t smem = grid_smem_bytes(tile_w);
  // the attribute is the kernel's ceiling for every launch: the largest dynamic shared memory
  // the device grants a block (launches then ask for their own tile's amount)
  const size_t ceiling = (size_t)grid_smem_optin() - 1024;
  if (smem > ceiling ||
      cudaFuncSetAttribute(net_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ceiling) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(kGridR * 8), 1, 1);
  cfg.blockDim = dim3(kGridThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kGridR;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, net_grid_kernel, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cached[dev][0] = tile_w;
  cached[dev][1] = clusters;
  return clusters;
}

struct GridLayout {
  size_t off_cnt, off_list, bytes;
  int ctas, slice;
};

static GridLayout grid_layout(int64_t n, int32_t tile_w) {
  GridLayout L{};
  const int64_t tiles = (n + tile_w - 1) / tile_w;
  L.ctas = (int)(tiles * kGridR);
  L.slice = tile_w / kGridR;
  L.off_cnt = 256;
  L.off_list = L.off_cnt + align_up(sizeof(int32_t) * 2 * (size_t)L.ctas, 256);
  L.bytes = L.off_list + sizeof(int32_t) * 2 * (size_t)L.ctas * (size_t)L.slice;
  return L;
}

struct JitLayout {
  size_t off_cnt, off_list, off_dge, off_dgi, bytes;
  int ctas, slice;
};

static JitLayout jit_layout(int64_t n) {
  JitLayout L{};
  L.ctas = std::min(device_sm_count(), kGridMaxCtas);
  int64_t slice = (n + L.ctas - 1) / L.ctas;
  slice = (slice + 31) / 32 * 32;
  L.slice = (int)std::max<int64_t>(slice, 32);
  L.off_cnt = 256;
  L.off_list = L.off_cnt + align_up(sizeof(int32_t) * 2 * (size_t)L.ctas, 256);
  L.off_dge = L.off_list + align_up(sizeof(int32_t) * 2 * (size_t)L.ctas * (size_t)L.slice, 256);
  L.off_dgi = L.off_dge + align_up(sizeof(float) * (size_t)n, 256);
  L.bytes = L.off_dgi + align_up(sizeof(float) * (size_t)n, 256);
  return L;
}

}  // namespace bp

using namespace bp;

static int g_grid_cooperative = -1;  // launch form of the last bp_net_run_grid

extern "C" {

int32_t bp_net_grid_cooperative(void) { return g_grid_cooperative; }

int32_t bp_net_grid_tile(int64_t n) {
  if (n <= 0) return 0;
  // the widest tile shared memory holds, then narrower ones while the clusters still fit
  const int max_tw = (int)(((size_t)grid_smem_optin() - 1024 - sizeof(int32_t) * (kGridMaxCtas + 1)) / sizeof(uint32_t)) -
                     kPlanPadSpan;
  int cap = max_tw / kGridTileAlign * kGridTileAlign;
  const int plan_cap = (int)kPlanMaxTileW / kGridTileAlign * kGridTileAlign;
  if (cap > plan_cap) cap = plan_cap;
  const int clusters = grid_max_clusters(cap);
  if (clusters <= 0) return 0;
  int64_t tw = (n + clusters - 1) / clusters;
  tw = (tw + kGridTileAlign - 1) / kGridTileAlign * kGridTileAlign;
  if (tw < kGridTileAlign) tw = kGridTileAlign;
  if (tw > cap) return 0;  // more tiles than clusters resident at once
  return (int32_t)tw;
}

size_t bp_net_grid_workspace_size(int64_t n, int32_t tile_w) {
  if (n <= 0 || tile_w <= 0) return 0;
  return grid_layout(n, tile_w).bytes;
}

bp_status bp_net_grid_error(const void* workspace, int32_t* error, bp_stream_t stream) {
  clear_error();
  BP_REQUIRE(workspace && error, BP_EINVAL, "net_grid_error: null pointer");
  BP_CUDA_TRY(cudaMemcpyAsync(error, static_cast<const char*>(workspace) + 8, sizeof(int32_t), cudaMemcpyDeviceToHost,
                              as_cuda(stream)));
  BP_CUDA_TRY(cudaStreamSynchronize(as_cuda(stream)));
  return BP_OK;
}

size_t bp_net_grid_jit_workspace_size(int64_t n) {
  if (n <= 0) return 0;
  return jit_layout(n).bytes;
}

bp_status bp_net_run_grid_jit(const bp_net_desc* desc, const uint32_t* seeds, int32_t clen, int32_t step0,
                              int32_t steps, float dt, void* workspace, size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(desc != nullptr && seeds != nullptr, BP_EINVAL, "net_run_grid_jit: null descriptor or seeds");
  const bp_net_desc& d = *desc;
  BP_REQUIRE(steps >= 0, BP_EINVAL, "net_run_grid_jit: negative steps");
  BP_REQUIRE(d.n > 0 && d.n_exc >= 0 && d.n_exc <= d.n, BP_EINVAL, "net_run_grid_jit: bad sizes n=%d n_exc=%d", d.n,
             d.n_exc);
  BP_REQUIRE((int64_t)d.n * 32 < INT32_MAX, BP_ENOTSUP,
             "net_run_grid_jit: %d neurons exceed the reference's int32 stream indexing", d.n);
  BP_REQUIRE(clen >= 1, BP_EINVAL, "net_run_grid_jit: conn_len must be >= 1 (got %d)", clen);
  BP_REQUIRE(d.ring == nullptr || d.ring_len == 0, BP_ENOTSUP, "net_run_grid_jit: synaptic delays are not supported");
  BP_REQUIRE(d.raster == nullptr, BP_ENOTSUP, "net_run_grid_jit: rasters are not supported");
  BP_REQUIRE(d.V && d.ge && d.gi && d.t_last && d.spike, BP_EINVAL, "net_run_grid_jit: null state array");
  const JitLayout L = jit_layout(d.n);
  BP_REQUIRE(workspace && workspace_bytes >= L.bytes, BP_ENOMEM, "net_run_grid_jit: workspace %zu < %zu",
             workspace_bytes, L.bytes);
  if (steps == 0) return BP_OK;
  static bool configured[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!configured[dev]) {
    int per_sm = 0;
    BP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, net_grid_jit_kernel, kGridThreads,
                                                              sizeof(int32_t) * (kGridMaxCtas + 1)));
    BP_REQUIRE(per_sm >= 1, BP_ENOTSUP, "net_run_grid_jit: the kernel cannot be resident");
    configured[dev] = true;
  }
  char* ws = static_cast<char*>(workspace);
  JitGridArgs g;
  g.bar = reinterpret_cast<uint32_t*>(ws);
  g.err = reinterpret_cast<int32_t*>(ws + 8);
  g.cnt = reinterpret_cast<int32_t*>(ws + L.off_cnt);
  g.list = reinterpret_cast<int32_t*>(ws + L.off_list);
  g.dge = reinterpret_cast<float*>(ws + L.off_dge);
  g.dgi = reinterpret_cast<float*>(ws + L.off_dgi);
  g.slice = L.slice;
  for (int k = 0; k < 4; ++k) g.seed[k] = seeds[k];
  const int32_t sh_e = (d.n_exc + 1) >> 5, sh_i = ((d.n - d.n_exc) + 1) >> 5;
  g.step_e = (uint32_t)(sh_e > 1 ? sh_e : 1);
  g.step_i = (uint32_t)(sh_i > 1 ? sh_i : 1);
  g.fm = make_fastmod((uint32_t)clen);
  BP_CUDA_TRY(cudaMemsetAsync(ws, 0, 8, st));  // barrier words (the error word is sticky)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)L.ctas, 1, 1);
  cfg.blockDim = dim3(kGridThreads, 1, 1);
  cfg.dynamicSmemBytes = sizeof(int32_t) * (size_t)(L.ctas + 1);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  ScopedKernelTimer tk(st);
  BP_CUDA_TRY(cudaLaunchKernelEx(&cfg, net_grid_jit_kernel, d, step0, steps, dt, g));
  return BP_OK;
}

bp_status bp_net_run_grid(const bp_net_desc* desc, int32_t step0, int32_t steps, float dt, void* workspace,
                          size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(desc != nullptr, BP_EINVAL, "net_run_grid: null descriptor");
  const bp_net_desc& d = *desc;
  BP_REQUIRE(steps >= 0, BP_EINVAL, "net_run_grid: negative steps");
  BP_REQUIRE(d.n > 0 && d.n_exc >= 0 && d.n_exc <= d.n, BP_EINVAL, "net_run_grid: bad sizes n=%d n_exc=%d", d.n,
             d.n_exc);
  BP_REQUIRE(d.tile_w > 0 && d.tile_w % kGridTileAlign == 0 && d.tile_w <= (int)kPlanMaxTileW, BP_EINVAL,
             "net_run_grid: tile_w %d must be a positive multiple of %d", d.tile_w, kGridTileAlign);
  BP_REQUIRE((int64_t)d.n_tiles == ((int64_t)d.n + d.tile_w - 1) / d.tile_w, BP_EINVAL,
             "net_run_grid: n_tiles %d does not match n=%d, tile_w=%d", d.n_tiles, d.n, d.tile_w);
  BP_REQUIRE(d.ring_len >= 0 && d.ring_len <= kGridMaxDelay, BP_ENOTSUP,
             "net_run_grid: %d delay steps exceed the %d the runner holds", d.ring_len, kGridMaxDelay);
  BP_REQUIRE(d.ring_len == 0 || d.ring != nullptr, BP_EINVAL, "net_run_grid: null spike history");
  BP_REQUIRE(d.raster == nullptr, BP_ENOTSUP, "net_run_grid: rasters are not supported");
  BP_REQUIRE(d.seg_off && d.idx && d.V && d.ge && d.gi && d.t_last && d.spike, BP_EINVAL,
             "net_run_grid: null state or plan array");
  const GridLayout L = grid_layout(d.n, d.tile_w);
  BP_REQUIRE(L.ctas <= kGridMaxCtas, BP_ENOTSUP, "net_run_grid: %d CTAs exceed %d", L.ctas, kGridMaxCtas);
  BP_REQUIRE(workspace && workspace_bytes >= L.bytes, BP_ENOMEM, "net_run_grid: workspace %zu < %zu",
             workspace_bytes, L.bytes);
  const int clusters = grid_max_clusters(d.tile_w);
  BP_REQUIRE(L.ctas / kGridR <= clusters, BP_ENOTSUP,
             "net_run_grid: %d tiles need %d clusters resident at once, the device holds %d", L.ctas / kGridR,
             L.ctas / kGridR, clusters);
  if (steps == 0) return BP_OK;
  char* ws = static_cast<char*>(workspace);
  GridArgs g;
  g.bar = reinterpret_cast<uint32_t*>(ws);
  g.err = reinterpret_cast<int32_t*>(ws + 8);
  g.cnt = reinterpret_cast<int32_t*>(ws + L.off_cnt);
  g.list = reinterpret_cast<int32_t*>(ws + L.off_list);
  g.slice = L.slice;
  BP_CUDA_TRY(cudaMemsetAsync(ws, 0, 8, st));  // barrier words (the error word is sticky)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)L.ctas, 1, 1);
  cfg.blockDim = dim3(kGridThreads, 1, 1);
  cfg.dynamicSmemBytes = grid_smem_bytes(d.tile_w);
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kGridR;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeCooperative;
  attr[1].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  ScopedKernelTimer tk(st);
  cudaError_t e = cudaLaunchKernelEx(&cfg, net_grid_kernel, d, step0, steps, dt, g);
  g_grid_cooperative = e == cudaSuccess ? 1 : 0;
  if (e != cudaSuccess) {
    // no cooperative scheduling with clusters here: the occupancy check above already showed
    // that every cluster is resident at once, and the barrier's waits are bounded
    cudaGetLastError();
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, net_grid_kernel, d, step0, steps, dt, g);
  }
  BP_CUDA_TRY(e);
  return BP_OK;
}

}  // extern "C"
