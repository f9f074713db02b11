// event_tiled.cu -- event.csrmv (transpose=1) on the column-tiled plan.
//
// Two kernels per call:
//   1. compact_blocked_kernel: the spike vector is cut into blocks of 4096 rows; each block
//      writes its active rows (ascending) to its own slot of `lists` and the number to
//      `counts` -- no atomics, nothing to reset between calls.
//   2. ecsr_t_tiled_kernel: a thread-block cluster of R CTAs owns one tile of tile_w output
//      columns.  CTA `rank` takes 1/R of the compaction blocks; for each active row it loads
//      the row's segment for its tile (tile-local uint16 indices in 8-byte chunks) and adds
//      into a shared-memory accumulator (uint32 counts for a homogeneous weight, float32
//      otherwise).  At the end the R accumulators of the cluster are summed through
//      distributed shared memory and every output column is written exactly once.
//
// The random scatter thus stays on-chip (shared-memory atomics), HBM sees the plan's
// segments once (2 B per event instead of the reference's 4 B int32 index) and the output
// once.  Reference semantics: brainpy/_src/math/event/_csr_matvec.py:321-339.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "common.cuh"
#include "compact.cuh"
#include "plan.cuh"
#include "timer.cuh"

namespace cg = cooperative_groups;

namespace bp {

constexpr int kCompactRows = 4096;  // rows per compaction block (256 threads x 16)
constexpr int kTiledThreads = 1024;
constexpr int kBlockGroup = 1024;   // compaction blocks scanned per group

// ---------------------------------------------------------------------------
// plan build: one CTA per row (grid-stride)
// ---------------------------------------------------------------------------
template <typename IdxT>
__global__ void __launch_bounds__(256) plan_build_kernel(const IdxT* __restrict__ indptr, const IdxT* __restrict__ indices,
                                                         const float* __restrict__ data, int64_t nnz, int64_t m,
                                                         int64_t n, int tile_w, int nt, uint64_t* __restrict__ row_start,
                                                         uint32_t* __restrict__ tile_off, uint16_t* __restrict__ idx,
                                                         float* __restrict__ w) {
  extern __shared__ uint32_t sm[];
  uint32_t* hist = sm;            // nt
  uint32_t* offs = sm + nt;       // nt + 1
  uint32_t* cursor = offs + nt + 1;  // nt
  const uint64_t per_row = 4ull * (uint64_t)nt + 4ull;
  for (int64_t row = blockIdx.x; row < m; row += gridDim.x) {
    int64_t b = (int64_t)indptr[row], e = (int64_t)indptr[row + 1];
    b = b < 0 ? 0 : (b > nnz ? nnz : b);
    e = e < b ? b : (e > nnz ? nnz : e);
    const uint64_t rs = (((uint64_t)b + 3ull) & ~3ull) + per_row * (uint64_t)row;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
      hist[t] = 0;
      cursor[t] = 0;
    }
    __syncthreads();
    for (int64_t j = b + threadIdx.x; j < e; j += blockDim.x) {
      int64_t c = (int64_t)indices[j];
      if (c >= 0 && c < n) atomicAdd(&hist[c / tile_w], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t acc = 0;
      for (int t = 0; t < nt; ++t) {
        offs[t] = acc;
        acc += (hist[t] + 3u) & ~3u;
      }
      offs[nt] = acc;
      row_start[row] = rs;
    }
    __syncthreads();
    for (int t = threadIdx.x; t <= nt; t += blockDim.x) tile_off[row * (int64_t)(nt + 1) + t] = offs[t];
    for (int64_t j = b + threadIdx.x; j < e; j += blockDim.x) {
      int64_t c = (int64_t)indices[j];
      if (c < 0 || c >= n) continue;
      int t = (int)(c / tile_w);
      uint32_t pos = atomicAdd(&cursor[t], 1u);
      uint64_t dst = rs + offs[t] + pos;
      idx[dst] = (uint16_t)(c - (int64_t)t * tile_w);
      if (w) w[dst] = data[j];
    }
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
      uint32_t h = hist[t], hp = (h + 3u) & ~3u;
      for (uint32_t p = h; p < hp; ++p) {
        uint64_t dst = rs + offs[t] + p;
        idx[dst] = kPadIndex;
        if (w) w[dst] = 0.0f;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// blocked compaction: block b handles rows [b*4096, (b+1)*4096)
// ---------------------------------------------------------------------------
template <int ET>
__global__ void __launch_bounds__(256) compact_blocked_kernel(const void* __restrict__ events, int64_t m,
                                                              int32_t* __restrict__ lists,
                                                              int32_t* __restrict__ counts) {
  // let the accumulation kernel launch and zero its shared memory while this grid runs;
  // it reads lists/counts only after cudaGridDependencySynchronize()
  cudaTriggerProgrammaticLaunchCompletion();
  const bool vec_ok = ((reinterpret_cast<uintptr_t>(events) & 15u) == 0);
  const int64_t blk0 = (int64_t)blockIdx.x * kCompactRows;
  const int64_t base = blk0 + (int64_t)threadIdx.x * 16;
  uint32_t mask = base < m ? load_event_mask16<ET>(events, base, m, vec_ok) : 0u;
  const int c = __popc(mask);
  const int lane = lane_id(), wid = threadIdx.x >> 5;
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  __shared__ int warp_tot[8];
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  int wpre = 0, total = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    wpre += k < wid ? warp_tot[k] : 0;
    total += warp_tot[k];
  }
  int pos = wpre + incl - c;
  int32_t* out = lists + blk0;
  while (mask) {
    int k = __ffs(mask) - 1;
    mask &= mask - 1;
    out[pos++] = (int32_t)(base + k);
  }
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// ---------------------------------------------------------------------------
// tiled accumulation
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint2 ld_stream_u2(const uint16_t* p) {
  return __ldcs(reinterpret_cast<const uint2*>(p));
}
__device__ __forceinline__ float4 ld_stream_f4(const float* p) { return __ldcs(reinterpret_cast<const float4*>(p)); }

// Accumulation modes of the tiled kernel:
//   kCount  homogeneous weight, events: uint32 event counts, out = (float)count * w
//   kWeight heterogeneous weights, events: float32 sum of w_ij
//   kRowVal homogeneous weight, dense vector x: float32 sum of x_i, out = w * sum
//   kWRow   heterogeneous weights, dense vector x: float32 sum of w_ij * x_i
enum { kCount = 0, kWeight = 1, kRowVal = 2, kWRow = 3 };

template <int MODE>
__device__ __forceinline__ void accumulate4(uint32_t* acc, uint2 v, float4 wv, float xv, uint32_t tile_w) {
  uint32_t x[4] = {v.x & 0xFFFFu, v.x >> 16, v.y & 0xFFFFu, v.y >> 16};
  float ww[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (x[q] < tile_w) {  // excludes the 0xFFFF padding
      if (MODE == kCount) atomicAdd(acc + x[q], 1u);
      else if (MODE == kWeight) atomicAdd(reinterpret_cast<float*>(acc) + x[q], ww[q]);
      else if (MODE == kRowVal) atomicAdd(reinterpret_cast<float*>(acc) + x[q], xv);
      else atomicAdd(reinterpret_cast<float*>(acc) + x[q], __fmul_rn(ww[q], xv));
    }
  }
}

struct TiledArgs {
  const uint64_t* row_start;
  const uint32_t* tile_off;
  const uint16_t* idx;
  const float* w;
  const int32_t* lists;
  const int32_t* counts;
  const float* w_homo;
  const float* row_val;  // dense vector for kRowVal / kWRow
  float* out;
  int64_t n;
  int32_t tile_w, n_tiles, nb, acc_words;
  int32_t vec_out;  // out is 16-byte aligned (tile_w is a multiple of 4)
};

// Warp-independent processing: after one CTA-wide prefix over this rank's compaction blocks,
// every warp walks "slices" of 32 active rows.  Lane l of a slice owns row 32k+l and fetches
// its segment descriptor (start, chunk count) for this CTA's tile; the row ids of slice k+2W
// and the descriptors of slice k+W are in flight while slice k is processed.  Inside a slice,
// groups of G lanes take one segment each (lane gl loads 8-byte chunk gl, 4 uint16 indices)
// and G segments are loaded back to back before any shared-memory atomic is issued.
template <int MODE, int G, int RND>
__global__ void __launch_bounds__(kTiledThreads, 1) ecsr_t_tiled_kernel(TiledArgs a) {
  constexpr bool HAS_W = (MODE == kWeight || MODE == kWRow);
  constexpr bool HAS_X = (MODE == kRowVal || MODE == kWRow);
  extern __shared__ uint4 smem_raw[];
  uint32_t* acc = reinterpret_cast<uint32_t*>(smem_raw);
  int* s_boff = reinterpret_cast<int*>(acc + a.acc_words);  // kBlockGroup + 1
  __shared__ int s_wsum[32];

  cg::cluster_group cluster = cg::this_cluster();
  const int R = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tile = blockIdx.x / R;
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;

  for (int i = tid; i < a.acc_words; i += nthr) acc[i] = 0u;

  const int b0 = (int)((int64_t)rank * a.nb / R), b1 = (int)((int64_t)(rank + 1) * a.nb / R);
  const uint64_t* __restrict__ row_start = a.row_start;
  const uint32_t* __restrict__ tile_off = a.tile_off;
  const int64_t toff_stride = a.n_tiles + 1;

  // the compaction kernel of this call may still be running (programmatic dependent launch)
  cudaGridDependencySynchronize();

  for (int g0 = b0; g0 < b1; g0 += kBlockGroup) {
    const int ng = min(kBlockGroup, b1 - g0);
    __syncthreads();  // s_boff of the previous group is no longer read
    int v = tid < ng ? a.counts[g0 + tid] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      int t = s_wsum[lane], ti = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, ti, o);
        if (lane >= o) ti += u;
      }
      s_wsum[lane] = ti - t;
    }
    __syncthreads();
    if (tid < ng) s_boff[tid] = s_wsum[warp] + incl - v;
    if (tid == ng - 1) s_boff[ng] = s_wsum[warp] + incl;
    __syncthreads();
    const int total = s_boff[ng];
    const int nslices = (total + 31) >> 5;

    // Lane-per-segment: in slice k (elements 32k .. 32k+31 of this rank's active-row list),
    // lane l owns row 32k+l and walks that row's segment for this tile on its own, so the
    // inner loop issues only global loads and shared-memory atomics (no shuffles).
    // row id of element g of this group's list; `blk` is the lane's running block hint
    auto fetch_row = [&](int k, int& blk) -> int32_t {
      const int g = (k << 5) + lane;
      if (k >= nslices || g >= total) return -1;
      while (s_boff[blk + 1] <= g) ++blk;  // blocks hold ~rate*4096 rows: a step or two
      return __ldg(a.lists + (int64_t)(g0 + blk) * kCompactRows + (g - s_boff[blk]));
    };
    auto block_of = [&](int g) -> int {
      int lo = 0, hi = ng;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (s_boff[mid] <= g) lo = mid;
        else hi = mid;
      }
      return lo;
    };
    auto fetch_desc = [&](int32_t row, uint32_t& st, uint32_t& nch, float& xv) {
      st = 0;
      nch = 0;
      xv = 0.0f;
      if (row >= 0) {
        if (HAS_X) xv = __ldg(a.row_val + row);
        const uint64_t rs = __ldg(row_start + row);
        const uint32_t* to = tile_off + (int64_t)row * toff_stride + tile;
        const uint32_t o0 = __ldg(to), o1 = __ldg(to + 1);
        st = (uint32_t)(rs + o0);
        nch = (o1 - o0) >> 2;
      }
    };

    int k = warp;
    int blk1 = block_of(min((k << 5) + lane, max(total - 1, 0)));
    uint32_t cst, cn;
    float cxv;
    fetch_desc(fetch_row(k, blk1), cst, cn, cxv);
    int blk2 = block_of(min(((k + nwarps) << 5) + lane, max(total - 1, 0)));
    int32_t row1 = fetch_row(k + nwarps, blk2);
    int blk3 = blk2;
    while (k < nslices) {
      uint32_t nst, nn;
      float nxv;
      fetch_desc(row1, nst, nn, nxv);  // slice k + W: in flight during slice k
      int32_t row2 = -1;
      if (k + 2 * nwarps < nslices) {
        blk3 = block_of(min(((k + 2 * nwarps) << 5) + lane, max(total - 1, 0)));
        row2 = fetch_row(k + 2 * nwarps, blk3);
      }
      // Groups of G lanes share a segment: group grp takes the segments of lanes
      // grp, grp + 32/G, ...; lane gl of the group loads chunks gl, gl + G, ... (RND rounds),
      // so one warp-wide load touches 32/G segments with G consecutive chunks each.  UB
      // segments are loaded before any of their atomics are issued.
      {
        constexpr int NG = 32 / G;
        constexpr int UBMAX = (HAS_W ? 4 : 8) / RND > 0 ? (HAS_W ? 4 : 8) / RND : 1;
        constexpr int UB = UBMAX > G ? G : UBMAX;
        const int grp = lane / G, gl = lane % G;
#pragma unroll 1
        for (int u0 = 0; u0 < G; u0 += UB) {
          uint2 vv[UB][RND];
          float4 wv[UB][RND];
          uint32_t st[UB], ln[UB];
          float xs[UB];
#pragma unroll
          for (int u = 0; u < UB; ++u) {
            const int j = grp + (u0 + u) * NG;
            st[u] = __shfl_sync(0xffffffffu, cst, j);
            ln[u] = __shfl_sync(0xffffffffu, cn, j);
            xs[u] = HAS_X ? __shfl_sync(0xffffffffu, cxv, j) : 0.0f;
#pragma unroll
            for (int r = 0; r < RND; ++r) {
              const uint32_t c = gl + r * G;
              if (c < ln[u]) {
                const uint32_t e = st[u] + 4u * c;
                vv[u][r] = ld_stream_u2(a.idx + e);
                if (HAS_W) wv[u][r] = ld_stream_f4(a.w + e);
              }
            }
          }
#pragma unroll
          for (int u = 0; u < UB; ++u)
#pragma unroll
            for (int r = 0; r < RND; ++r)
              if (gl + r * G < ln[u])
                accumulate4<MODE>(acc, vv[u][r], HAS_W ? wv[u][r] : make_float4(0, 0, 0, 0), xs[u], a.tile_w);
          // chunks beyond RND*G (long segments): rare, plain loop
#pragma unroll
          for (int u = 0; u < UB; ++u) {
            for (uint32_t c = gl + RND * G; c < ln[u]; c += G) {
              const uint32_t e = st[u] + 4u * c;
              const uint2 x = ld_stream_u2(a.idx + e);
              const float4 y = HAS_W ? ld_stream_f4(a.w + e) : make_float4(0, 0, 0, 0);
              accumulate4<MODE>(acc, x, y, xs[u], a.tile_w);
            }
          }
        }
      }
      cst = nst;
      cn = nn;
      cxv = nxv;
      row1 = row2;
      k += nwarps;
    }
  }

  // ---- reduce the cluster's accumulators and write the tile
  cluster.sync();
  const int slice = a.acc_words / R;  // multiple of 4
  const int c0 = rank * slice;
  const float w = (MODE == kCount || MODE == kRowVal) ? __ldg(a.w_homo) : 0.0f;
  const int64_t col_base = (int64_t)tile * a.tile_w;
  for (int c = c0 + 4 * tid; c < c0 + slice; c += 4 * nthr) {
    float o[4];
    if (MODE == kCount) {
      uint4 s = make_uint4(0, 0, 0, 0);
      for (int r = 0; r < R; ++r) {
        const uint4 x = *reinterpret_cast<const uint4*>(cluster.map_shared_rank(acc, r) + c);
        s.x += x.x;
        s.y += x.y;
        s.z += x.z;
        s.w += x.w;
      }
      o[0] = (float)s.x * w;
      o[1] = (float)s.y * w;
      o[2] = (float)s.z * w;
      o[3] = (float)s.w * w;
    } else {
      float4 s = make_float4(0, 0, 0, 0);
      for (int r = 0; r < R; ++r) {
        const float4 x = *reinterpret_cast<const float4*>(cluster.map_shared_rank(acc, r) + c);
        s.x += x.x;
        s.y += x.y;
        s.z += x.z;
        s.w += x.w;
      }
      if (MODE == kRowVal) {
        s.x = __fmul_rn(w, s.x);
        s.y = __fmul_rn(w, s.y);
        s.z = __fmul_rn(w, s.z);
        s.w = __fmul_rn(w, s.w);
      }
      o[0] = s.x;
      o[1] = s.y;
      o[2] = s.z;
      o[3] = s.w;
    }
    const int64_t gc = col_base + c;
    if (a.vec_out && c + 3 < a.tile_w && gc + 3 < a.n) {
      *reinterpret_cast<float4*>(a.out + gc) = make_float4(o[0], o[1], o[2], o[3]);
    } else {
      for (int q = 0; q < 4; ++q)
        if (c + q < a.tile_w && gc + q < a.n) a.out[gc + q] = o[q];
    }
  }
  cluster.sync();
}

static size_t tiled_smem_bytes(int acc_words) {
  return sizeof(uint32_t) * (size_t)acc_words + sizeof(int) * (kBlockGroup + 1);
}

static int acc_words_for(int tile_w, int R) {
  int q = 4 * R;
  return (tile_w + q - 1) / q * q;
}

template <int MODE, int G, int RND>
static bp_status launch_tiled_g(const TiledArgs& a, int R, cudaStream_t st) {
  auto kfn = ecsr_t_tiled_kernel<MODE, G, RND>;
  const size_t smem = tiled_smem_bytes(a.acc_words);
  static thread_local size_t configured[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (configured[dev] < smem) {
    BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    configured[dev] = smem;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(a.n_tiles * R), 1, 1);
  cfg.blockDim = dim3(kTiledThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)R;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  BP_CUDA_TRY(cudaLaunchKernelEx(&cfg, kfn, a));
  return BP_OK;
}

// (lanes per segment, chunk rounds) from the mean segment length in 8-byte chunks; the
// environment variable BPGPU_TILED_GROUP=G,RND overrides (tuning).
static void choose_group(double chunks, int& G, int& RND) {
  if (chunks <= 1.5) { G = 1; RND = 2; }
  else if (chunks <= 4.5) { G = 2; RND = 2; }
  else if (chunks <= 10.0) { G = 4; RND = 2; }
  else if (chunks <= 14.0) { G = 4; RND = 3; }
  else { G = 8; RND = 2; }
  static int env_g = -1, env_r = -1;
  if (env_g < 0) {
    env_g = 0;
    const char* e = getenv("BPGPU_TILED_GROUP");
    if (e) sscanf(e, "%d,%d", &env_g, &env_r);
  }
  if (env_g > 0) {
    G = env_g;
    RND = env_r > 0 ? env_r : 2;
  }
}

template <int MODE>
static bp_status launch_tiled(const TiledArgs& a, int R, double chunks, cudaStream_t st) {
  int G, RND;
  choose_group(chunks, G, RND);
  if (G == 1) return launch_tiled_g<MODE, 1, 2>(a, R, st);
  if (G == 2) return launch_tiled_g<MODE, 2, 2>(a, R, st);
  if (G == 4 && RND == 2) return launch_tiled_g<MODE, 4, 2>(a, R, st);
  if (G == 4) return launch_tiled_g<MODE, 4, 3>(a, R, st);
  if (G == 8 && RND == 1) return launch_tiled_g<MODE, 8, 1>(a, R, st);
  if (G == 8) return launch_tiled_g<MODE, 8, 2>(a, R, st);
  return launch_tiled_g<MODE, 16, 1>(a, R, st);
}

template <int ET>
static bp_status launch_compact_blocked(const void* events, int64_t m, int32_t* lists, int32_t* counts,
                                        cudaStream_t st) {
  int nb = (int)((m + kCompactRows - 1) / kCompactRows);
  compact_blocked_kernel<ET><<<nb, 256, 0, st>>>(events, m, lists, counts);
  return check_launch("compact_blocked_kernel");
}

static bp_status compact_blocked(const void* events, bp_etype et, int64_t m, int32_t* lists, int32_t* counts,
                                 cudaStream_t st) {
  switch (et) {
    case BP_EV_BOOL: return launch_compact_blocked<BP_EV_BOOL>(events, m, lists, counts, st);
    case BP_EV_F32_POS: return launch_compact_blocked<BP_EV_F32_POS>(events, m, lists, counts, st);
    case BP_EV_F32_NZ: return launch_compact_blocked<BP_EV_F32_NZ>(events, m, lists, counts, st);
  }
  return BP_EINVAL;
}

static int max_active_clusters(int R, size_t smem) {
  auto kfn = ecsr_t_tiled_kernel<kCount, 4, 3>;
  if (cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(R * 64), 1, 1);
  cfg.blockDim = dim3(kTiledThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)R;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int num = 0;
  if (cudaOccupancyMaxActiveClusters(&num, kfn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return num;
}

static int max_smem_optin() {
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

}  // namespace bp

using namespace bp;

extern "C" {

int32_t bp_csr_plan_default_tile(int64_t n, int32_t cluster) {
  if (n <= 0) return 0;
  if (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8) cluster = 4;
  const int64_t cap_words = (int64_t)(max_smem_optin() - 4 * (kBlockGroup + 1) - 1024) / 4;
  const int64_t cap_tw = std::min<int64_t>(cap_words / 64 * 64, kPlanMaxTileW / 64 * 64);
  // how many clusters of `cluster` CTAs (one CTA per SM) can be resident at once
  int clusters = max_active_clusters(cluster, tiled_smem_bytes((int)cap_tw));
  if (clusters < 1) clusters = std::max(1, device_sm_count() / cluster);
  int64_t tw = (n + clusters - 1) / clusters;
  tw = (tw + 63) / 64 * 64;
  if (tw > cap_tw) tw = cap_tw;
  if (tw < 64) tw = 64;
  return (int32_t)tw;
}

size_t bp_csr_plan_bytes(int64_t m, int64_t n, int64_t nnz, int32_t heter, int32_t tile_w) {
  if (m < 0 || n <= 0 || nnz < 0 || tile_w <= 0) return 0;
  int64_t nt = (n + tile_w - 1) / tile_w;
  return plan_layout(m, nnz, (int32_t)nt, heter != 0).total;
}

bp_status bp_csr_plan_build(const float* data, int64_t ndata, const void* indices, const void* indptr,
                            bp_itype itype, int64_t nnz, int64_t m, int64_t n, int32_t tile_w, void* mem,
                            size_t bytes, bp_csr_plan* plan_out, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(plan_out != nullptr, BP_EINVAL, "csr_plan_build: null plan_out");
  BP_REQUIRE(m >= 0 && n > 0 && nnz >= 0, BP_EINVAL, "csr_plan_build: bad sizes m=%lld n=%lld nnz=%lld",
             (long long)m, (long long)n, (long long)nnz);
  BP_REQUIRE(m <= INT32_MAX && n <= INT32_MAX, BP_ENOTSUP, "csr_plan_build: dimensions beyond int32 range");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "csr_plan_build: bad index type");
  BP_REQUIRE(tile_w >= 64 && tile_w <= kPlanMaxTileW && tile_w % 4 == 0, BP_EINVAL,
             "csr_plan_build: tile_w %d must be a multiple of 4 in [64, %d]", tile_w, kPlanMaxTileW);
  const int64_t nt = (n + tile_w - 1) / tile_w;
  BP_REQUIRE(nt <= kPlanMaxTiles, BP_ENOTSUP, "csr_plan_build: %lld tiles exceed %d", (long long)nt, kPlanMaxTiles);
  const bool heter = data != nullptr && ndata > 1;
  BP_REQUIRE(!heter || ndata == nnz, BP_ESHAPE, "csr_plan_build: data size %lld != nnz %lld", (long long)ndata,
             (long long)nnz);
  PlanLayout L = plan_layout(m, nnz, (int32_t)nt, heter);
  BP_REQUIRE(L.entries < (1ull << 32), BP_ENOTSUP, "csr_plan_build: %llu padded entries exceed 2^32",
             (unsigned long long)L.entries);
  BP_REQUIRE(mem != nullptr && bytes >= L.total, BP_ENOMEM, "csr_plan_build: memory %zu < %zu", bytes, L.total);
  BP_REQUIRE(m == 0 || (indices && indptr) || nnz == 0, BP_EINVAL, "csr_plan_build: null indices/indptr");
  bp_csr_plan p = {};
  p.m = m;
  p.n = n;
  p.nnz = nnz;
  p.tile_w = tile_w;
  p.n_tiles = (int32_t)nt;
  p.heter = heter ? 1 : 0;
  p.entries = L.entries;
  p.mem = mem;
  p.bytes = bytes;
  char* base = static_cast<char*>(mem);
  uint64_t* rs = reinterpret_cast<uint64_t*>(base + L.off_row_start);
  uint32_t* toff = reinterpret_cast<uint32_t*>(base + L.off_tile_off);
  uint16_t* idx = reinterpret_cast<uint16_t*>(base + L.off_idx);
  float* w = heter ? reinterpret_cast<float*>(base + L.off_w) : nullptr;
  if (m > 0) {
    if (nnz == 0) {
      BP_CUDA_TRY(cudaMemsetAsync(toff, 0, sizeof(uint32_t) * (size_t)m * (size_t)(nt + 1), st));
      BP_CUDA_TRY(cudaMemsetAsync(rs, 0, sizeof(uint64_t) * (size_t)m, st));
    } else {
      int grid = (int)std::min<int64_t>(m, (int64_t)device_sm_count() * 16);
      size_t smem = sizeof(uint32_t) * (size_t)(3 * nt + 1);
      if (itype == BP_I32)
        plan_build_kernel<int32_t><<<grid, 256, smem, st>>>(static_cast<const int32_t*>(indptr),
                                                             static_cast<const int32_t*>(indices), data, nnz, m, n,
                                                             tile_w, (int)nt, rs, toff, idx, w);
      else
        plan_build_kernel<int64_t><<<grid, 256, smem, st>>>(static_cast<const int64_t*>(indptr),
                                                             static_cast<const int64_t*>(indices), data, nnz, m, n,
                                                             tile_w, (int)nt, rs, toff, idx, w);
      bp_status s = check_launch("plan_build_kernel");
      if (s != BP_OK) return s;
    }
  }
  *plan_out = p;
  return BP_OK;
}

bp_status bp_csr_plan_arrays(const bp_csr_plan* plan, const uint64_t** row_start, const uint32_t** tile_off,
                             const uint16_t** idx, const float** w) {
  clear_error();
  BP_REQUIRE(plan != nullptr && plan->mem != nullptr, BP_EINVAL, "csr_plan_arrays: null plan");
  PlanView v = plan_view(plan);
  if (row_start) *row_start = v.row_start;
  if (tile_off) *tile_off = v.tile_off;
  if (idx) *idx = v.idx;
  if (w) *w = v.w;
  return BP_OK;
}

size_t bp_event_csrmv_planned_workspace_size(const bp_csr_plan* plan) {
  if (!plan || plan->m <= 0) return 256;
  int64_t nb = (plan->m + kCompactRows - 1) / kCompactRows;
  return align_up(sizeof(int32_t) * (size_t)nb * kCompactRows, 256) + align_up(sizeof(int32_t) * (size_t)nb, 256);
}

bp_status bp_event_csrmv_planned(const bp_csr_plan* plan, const float* w_homo, const void* events, bp_etype etype,
                                 float* out, int32_t cluster, void* workspace, size_t workspace_bytes,
                                 bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(plan != nullptr && plan->mem != nullptr, BP_EINVAL, "event_csrmv_planned: null plan");
  BP_REQUIRE(etype >= BP_EV_BOOL && etype <= BP_EV_F32_NZ, BP_EDTYPE, "event_csrmv_planned: bad event type %d",
             (int)etype);
  if (cluster == 0) cluster = 4;
  BP_REQUIRE(cluster == 1 || cluster == 2 || cluster == 4 || cluster == 8, BP_EINVAL,
             "event_csrmv_planned: cluster must be 1, 2, 4 or 8 (got %d)", cluster);
  const int64_t m = plan->m, n = plan->n;
  if (n == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "event_csrmv_planned: null out");
  if (m == 0 || plan->nnz == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n, st));
    return BP_OK;
  }
  BP_REQUIRE(events != nullptr, BP_EINVAL, "event_csrmv_planned: null events");
  const bool homo = plan->heter == 0;
  BP_REQUIRE(!homo || w_homo != nullptr, BP_EINVAL, "event_csrmv_planned: homogeneous plan needs w_homo");
  BP_REQUIRE(workspace && workspace_bytes >= bp_event_csrmv_planned_workspace_size(plan), BP_ENOMEM,
             "event_csrmv_planned: workspace %zu < %zu", workspace_bytes,
             bp_event_csrmv_planned_workspace_size(plan));
  const int acc_words = acc_words_for(plan->tile_w, cluster);
  BP_REQUIRE(tiled_smem_bytes(acc_words) <= (size_t)max_smem_optin(), BP_ENOTSUP,
             "event_csrmv_planned: tile of %d columns does not fit shared memory", plan->tile_w);
  const int nb = (int)((m + kCompactRows - 1) / kCompactRows);
  int32_t* lists = static_cast<int32_t*>(workspace);
  int32_t* counts = reinterpret_cast<int32_t*>(static_cast<char*>(workspace) +
                                               align_up(sizeof(int32_t) * (size_t)nb * kCompactRows, 256));
  ScopedKernelTimer tk(st);  // brackets both kernels of the call
  bp_status s = compact_blocked(events, etype, m, lists, counts, st);
  if (s != BP_OK) return s;
  PlanView v = plan_view(plan);
  TiledArgs a;
  a.row_start = v.row_start;
  a.tile_off = v.tile_off;
  a.idx = v.idx;
  a.w = v.w;
  a.lists = lists;
  a.counts = counts;
  a.w_homo = w_homo;
  a.row_val = nullptr;
  a.out = out;
  a.n = n;
  a.tile_w = plan->tile_w;
  a.n_tiles = plan->n_tiles;
  a.nb = nb;
  a.acc_words = acc_words;
  a.vec_out = ((reinterpret_cast<uintptr_t>(out) & 15u) == 0) ? 1 : 0;
  const double chunks = ((double)plan->nnz / (double)m / (double)plan->n_tiles + 1.5) / 4.0;
  s = homo ? launch_tiled<kCount>(a, cluster, chunks, st) : launch_tiled<kWeight>(a, cluster, chunks, st);
  return s;
}

}  // extern "C"

extern "C" {

// sparse.csrmv, transpose=1, on a plan: out[j] = sum_i A[i, j] * vec[i].  Rows with vec[i] == 0
// contribute nothing and are skipped by the compaction (the dense vector is treated as
// events under the != 0 rule); the others carry their value into the tile accumulation.
bp_status bp_csrmv_planned(const bp_csr_plan* plan, const float* w_homo, const float* vec, float* out,
                           int32_t cluster, void* workspace, size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(plan != nullptr && plan->mem != nullptr, BP_EINVAL, "csrmv_planned: null plan");
  if (cluster == 0) cluster = 4;
  BP_REQUIRE(cluster == 1 || cluster == 2 || cluster == 4 || cluster == 8, BP_EINVAL,
             "csrmv_planned: cluster must be 1, 2, 4 or 8 (got %d)", cluster);
  const int64_t m = plan->m, n = plan->n;
  if (n == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "csrmv_planned: null out");
  if (m == 0 || plan->nnz == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n, st));
    return BP_OK;
  }
  BP_REQUIRE(vec != nullptr, BP_EINVAL, "csrmv_planned: null vector");
  const bool homo = plan->heter == 0;
  BP_REQUIRE(!homo || w_homo != nullptr, BP_EINVAL, "csrmv_planned: homogeneous plan needs w_homo");
  BP_REQUIRE(workspace && workspace_bytes >= bp_event_csrmv_planned_workspace_size(plan), BP_ENOMEM,
             "csrmv_planned: workspace %zu < %zu", workspace_bytes, bp_event_csrmv_planned_workspace_size(plan));
  const int acc_words = acc_words_for(plan->tile_w, cluster);
  BP_REQUIRE(tiled_smem_bytes(acc_words) <= (size_t)max_smem_optin(), BP_ENOTSUP,
             "csrmv_planned: tile of %d columns does not fit shared memory", plan->tile_w);
  const int nb = (int)((m + kCompactRows - 1) / kCompactRows);
  int32_t* lists = static_cast<int32_t*>(workspace);
  int32_t* counts = reinterpret_cast<int32_t*>(static_cast<char*>(workspace) +
                                               align_up(sizeof(int32_t) * (size_t)nb * kCompactRows, 256));
  ScopedKernelTimer tk(st);
  bp_status s = compact_blocked(vec, BP_EV_F32_NZ, m, lists, counts, st);
  if (s != BP_OK) return s;
  PlanView v = plan_view(plan);
  TiledArgs a;
  a.row_start = v.row_start;
  a.tile_off = v.tile_off;
  a.idx = v.idx;
  a.w = v.w;
  a.lists = lists;
  a.counts = counts;
  a.w_homo = w_homo;
  a.row_val = vec;
  a.out = out;
  a.n = n;
  a.tile_w = plan->tile_w;
  a.n_tiles = plan->n_tiles;
  a.nb = nb;
  a.acc_words = acc_words;
  a.vec_out = ((reinterpret_cast<uintptr_t>(out) & 15u) == 0) ? 1 : 0;
  const double chunks = ((double)plan->nnz / (double)m / (double)plan->n_tiles + 1.5) / 4.0;
  return homo ? launch_tiled<kRowVal>(a, cluster, chunks, st) : launch_tiled<kWRow>(a, cluster, chunks, st);
}

}  // extern "C"
