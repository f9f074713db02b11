// event_tiled.cu -- event.csrmv (transpose=1) on the column-tiled plan.
//
// Two kernels per call:
//   1. compact_blocked_kernel: the spike vector is cut into blocks of 4096 rows; each block
//      writes its active rows (ascending) to its own slot of `lists` and the number to
//      `counts` -- no atomics, nothing to reset between calls.
//   2. ecsr_t_tiled_kernel: a thread-block cluster of R CTAs owns one tile of tile_w output
//      columns.  CTA `rank` takes 1/R of the compaction blocks; for each active row it loads
//      the row's segment for its tile (16-byte chunks of 8 tile-local uint16 indices) and adds
//      into a shared-memory accumulator (uint32 counts for a homogeneous weight, float32
//      otherwise), with the next rows' segments in flight.  At the end the R
//      accumulators of the cluster are summed through distributed shared memory and every
//      output column is written exactly once.
//
// The random scatter thus stays on-chip (shared-memory atomics), HBM sees the plan's
// segments once (2 B per event instead of the reference's 4 B int32 index) and the output
// once.  Reference semantics: brainpy/_src/math/event/_csr_matvec.py:321-339.
#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>
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
constexpr size_t kStaticSmemReserve = 1024;  // the kernel's static shared variables

// ---------------------------------------------------------------------------
// plan build: one CTA per row (grid-stride)
// ---------------------------------------------------------------------------
template <typename IdxT>
__global__ void __launch_bounds__(256) plan_build_kernel(const IdxT* __restrict__ indptr, const IdxT* __restrict__ indices,
                                                         const float* __restrict__ data, int64_t nnz, int64_t m,
                                                         int64_t n, int tile_w, int nt, uint32_t* __restrict__ seg_off,
                                                         uint16_t* __restrict__ idx, float* __restrict__ w,
                                                         uint32_t* __restrict__ meta) {
  extern __shared__ uint32_t sm[];
  uint32_t* hist = sm;               // nt
  uint32_t* offs = sm + nt;          // nt + 1
  uint32_t* cursor = offs + nt + 1;  // nt
  uint32_t* tab = cursor + nt;       // 2 * kPlanDupCheckMax: open-addressing set of a row's columns
  __shared__ int s_dup;
  const uint64_t per_row = 8ull * (uint64_t)nt + 8ull;
  for (int i = threadIdx.x; i < 2 * kPlanDupCheckMax; i += blockDim.x) tab[i] = 0xFFFFFFFFu;
  for (int64_t row = blockIdx.x; row < m; row += gridDim.x) {
    int64_t b = (int64_t)indptr[row], e = (int64_t)indptr[row + 1];
    b = b < 0 ? 0 : (b > nnz ? nnz : b);
    e = e < b ? b : (e > nnz ? nnz : e);
    const uint64_t rs = (((uint64_t)b + 7ull) & ~7ull) + per_row * (uint64_t)row;  // a multiple of 8
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
      hist[t] = 0;
      cursor[t] = 0;
    }
    if (threadIdx.x == 0) {
      s_dup = 0;
      atomicMax(&meta[1], (uint32_t)(e - b));
    }
    __syncthreads();
    // repeated columns: every in-range column of the row goes into a set of at least twice the
    // row's length (a power of two); a column found already present is a repeat.  Rows longer
    // than kPlanDupCheckMax are not checked and count as having repeats.
    if (e - b > kPlanDupCheckMax) {
      if (threadIdx.x == 0) meta[0] = 0u;
    } else if (e - b > 1) {
      uint32_t tsz = 64;
      while (tsz < 2u * (uint32_t)(e - b)) tsz <<= 1;
      const uint32_t mask = tsz - 1;
      for (int64_t j = b + threadIdx.x; j < e; j += blockDim.x) {
        const int64_t c = (int64_t)indices[j];
        if (c < 0 || c >= n) continue;
        uint32_t h = ((uint32_t)c * 2654435761u) & mask;
        for (uint32_t probe = 0; probe < tsz; ++probe, h = (h + 1) & mask) {
          const uint32_t old = atomicCAS(&tab[h], 0xFFFFFFFFu, (uint32_t)c);
          if (old == 0xFFFFFFFFu) break;
          if (old == (uint32_t)c) {
            s_dup = 1;
            break;
          }
        }
      }
      __syncthreads();
      if (threadIdx.x == 0 && s_dup) meta[0] = 0u;
      for (uint32_t i = threadIdx.x; i < tsz; i += blockDim.x) tab[i] = 0xFFFFFFFFu;
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
        acc += (hist[t] + 7u) & ~7u;
      }
      offs[nt] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t <= nt; t += blockDim.x)
      seg_off[row * (int64_t)(nt + 1) + t] = (uint32_t)((rs + offs[t]) >> 3);
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
      uint32_t h = hist[t], hp = (h + 7u) & ~7u;
      for (uint32_t p = h; p < hp; ++p) {
        uint64_t dst = rs + offs[t] + p;
        idx[dst] = (uint16_t)(tile_w + (((dst >> 3) & 3u) << 3) + (dst & 7u));  // a pad index past the tile
        if (w) w[dst] = 0.0f;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// blocked compaction: block b handles rows [b*4096, (b+1)*4096)
// ---------------------------------------------------------------------------
template <int ET, bool BATCH>
__global__ void __launch_bounds__(256) compact_blocked_kernel(const void* __restrict__ events, int64_t m,
                                                              int32_t* __restrict__ lists,
                                                              int32_t* __restrict__ counts) {
  // let the accumulation kernel launch and zero its shared memory while this grid runs;
  // it reads lists/counts only after cudaGridDependencySynchronize()
  cudaTriggerProgrammaticLaunchCompletion();
  // vector blockIdx.y of a batch: rows of m events, lists of gridDim.x * 4096, counts of gridDim.x
  // (a separate instantiation: the offsets cost measurable time in the single-vector call)
  if (BATCH) {
    const int64_t b = blockIdx.y;
    events = static_cast<const char*>(events) + b * m * (ET == BP_EV_BOOL ? 1 : 4);
    lists += b * (int64_t)gridDim.x * kCompactRows;
    counts += b * (int64_t)gridDim.x;
  }
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
// Accumulation modes:
//   kCount  homogeneous weight, events: uint32 count per column, out = (float)count * w
//   kWeight heterogeneous weights, events: float32 sum of w_ij
//   kRowVal homogeneous weight, dense vector x: float32 sum of x_i, out = w * sum
//   kWRow   heterogeneous weights, dense vector x: float32 sum of w_ij * x_i
//   kFix    heterogeneous weights held as int32 fixed point (w * 2^k, a fixed-weight plan),
//           events: exact integer sums, out = (float)sum * 2^-k
//   kFix24  kFix with the integer weights stored in 24 bits (40-byte chunk records)
enum { kCount = 0, kWeight = 1, kRowVal = 2, kWRow = 3, kFix = 4, kFix24 = 5 };

__host__ __device__ constexpr bool fixed_mode(int mode) { return mode == kFix || mode == kFix24; }
__host__ __device__ constexpr bool weighted_mode(int mode) {
  return mode == kWeight || mode == kWRow || fixed_mode(mode);
}

// Threads of a tiled CTA: 1024 (64 registers a thread), except the per-synapse-weight modes
// with two chunk rounds, whose double-buffered 40- or 48-byte chunks need more than 64
// registers: 768 threads (80 registers) there.
template <int MODE, int RND>
constexpr int tiled_threads() {
  return (weighted_mode(MODE) && RND >= 2) ? 768 : kTiledThreads;
}

// Shared-memory reductions issued under a predicate (no branch): entries with index >= lim
// are skipped -- the padding (index tile_w), and every entry of a chunk given lim = 0.
__device__ __forceinline__ void red_if(uint32_t x, uint32_t lim, uint32_t addr, uint32_t v) {
  asm volatile("{\n\t.reg .pred p;\n\tsetp.lt.u32 p, %0, %1;\n\t@p red.shared.add.u32 [%2], %3;\n\t}" ::"r"(x),
               "r"(lim), "r"(addr), "r"(v));
}
__device__ __forceinline__ void red_if(uint32_t x, uint32_t lim, uint32_t addr, float v) {
  asm volatile("{\n\t.reg .pred p;\n\tsetp.lt.u32 p, %0, %1;\n\t@p red.shared.add.f32 [%2], %3;\n\t}" ::"r"(x),
               "r"(lim), "r"(addr), "f"(v));
}

// Integer weight j (0..7) of a 40-byte chunk record: the low 16 bits from lo (two a word), the
// high byte from hi (four a word), sign-extended from bit 23 by the byte permute.
template <int J>
__device__ __forceinline__ uint32_t fix24_weight(const uint32_t lo[4], const uint32_t hi[2]) {
  constexpr uint32_t b0 = 2u * (J & 1), b2 = 4u + (J & 3);
  constexpr uint32_t sel = b0 | ((b0 + 1u) << 4) | (b2 << 8) | ((8u | b2) << 12);  // 8: replicate the sign
  uint32_t q;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(q) : "r"(lo[J >> 1]), "r"(hi[J >> 2]), "n"(sel));
  return q;
}

// Adds the 8 entries of one chunk (tile-local indices) into the accumulator at shared-memory
// address acc_s.
template <int MODE>
__device__ __forceinline__ void accumulate8(uint32_t acc_s, uint4 v, float4 w0, float4 w1, float xv, uint32_t lim) {
  const uint32_t x[8] = {v.x & 0xFFFFu, v.x >> 16, v.y & 0xFFFFu, v.y >> 16,
                         v.z & 0xFFFFu, v.z >> 16, v.w & 0xFFFFu, v.w >> 16};
  const float ww[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
  if (MODE == kFix24) {  // w0: the 16-bit halves, w1.x / w1.y: the high bytes
    const uint32_t lo[4] = {__float_as_uint(w0.x), __float_as_uint(w0.y), __float_as_uint(w0.z),
                            __float_as_uint(w0.w)};
    const uint32_t hi[2] = {__float_as_uint(w1.x), __float_as_uint(w1.y)};
    const uint32_t qq[8] = {fix24_weight<0>(lo, hi), fix24_weight<1>(lo, hi), fix24_weight<2>(lo, hi),
                            fix24_weight<3>(lo, hi), fix24_weight<4>(lo, hi), fix24_weight<5>(lo, hi),
                            fix24_weight<6>(lo, hi), fix24_weight<7>(lo, hi)};
#pragma unroll
    for (int q = 0; q < 8; ++q) asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(acc_s + 4u * x[q]), "r"(qq[q]));
    return;
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const uint32_t ad = acc_s + 4u * x[q];
    // counts: every entry adds, pads to the dummy words past the tile (lanes without a chunk
    // carry pads too), which saves the predicate (about half the add's instructions).  Float
    // adds stay predicated: unpredicated, the pads of every warp meet on the 32 dummy words,
    // and contended float adds to shared memory cost far more than the predicate saves
    // (measured: 77 us against 60 us per call at N = 1e6, fan-out 1000, 2 % events).
    if (MODE == kCount) asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(ad));
    else if (MODE == kFix) asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(ad), "r"(__float_as_uint(ww[q])));
    else if (MODE == kWeight) red_if(x[q], lim, ad, ww[q]);
    else if (MODE == kRowVal) red_if(x[q], lim, ad, xv);
    else red_if(x[q], lim, ad, __fmul_rn(ww[q], xv));
  }
}

__device__ __forceinline__ uint4 ld_stream_u4(const uint16_t* p) { return __ldcs(reinterpret_cast<const uint4*>(p)); }

// 40-byte chunk records of a fixed-weight plan whose integer weights fit in 24 bits: chunk c at
// byte 40c holds its 8 tile-local indices (16 bytes), the low 16 bits of its 8 weights (16 bytes)
// and their high bytes (8 bytes).  An even chunk starts on a 16-byte boundary and stores them in
// that order; an odd chunk starts 8 bytes past one and stores the high bytes first.  Either way
// the indices and the low halves are 16-byte loads and the high bytes an 8-byte load.
__device__ __forceinline__ void fix24_load(const uint4* fx, uint64_t c, uint4& idx, float4& lo, float4& hi) {
  const unsigned char* rec = reinterpret_cast<const unsigned char*>(fx) + 40ull * c;
  const uint32_t odd = (uint32_t)c & 1u;
  idx = __ldcs(reinterpret_cast<const uint4*>(rec + 8u * odd));
  lo = __ldcs(reinterpret_cast<const float4*>(rec + 16u + 8u * odd));
  const float2 h = __ldcs(reinterpret_cast<const float2*>(rec + 32u - 32u * odd));
  hi = make_float4(h.x, h.y, 0.0f, 0.0f);
}
__device__ __forceinline__ float4 ld_stream_f4(const float* p) { return __ldcs(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

struct TiledArgs {
  const uint32_t* seg_off;
  const uint16_t* idx;
  const float* w;
  const int32_t* lists;
  const int32_t* counts;
  const float* w_homo;
  const float* row_val;  // dense vector for kRowVal / kWRow
  const uint32_t* meta;  // plan meta ([2]: the fixed-point exponent of kFix / kFix24)
  const uint4* fx;       // kFix: chunk c's 8 indices and 8 integer weights at fx[3c .. 3c + 2];
                         // kFix24: chunk c's 40-byte record at byte 40c (fix24_record)
  float* out;
  int64_t m, n;  // a batch of vectors: row_val rows of m, out rows of n
  int32_t tile_w, n_tiles, nb, acc_words;
  int32_t batch;    // vectors per launch: gridDim.y
  int32_t variant;  // the plan's chosen kernel variant (0: from the segment length)
  int32_t vec_out;  // every vector's out row is 16-byte aligned (tile_w is a multiple of 4)
};

// Warp-independent processing: after one CTA-wide prefix over this rank's compaction blocks,
// every warp walks "slices" of 32 active rows (slices warp, warp + W, ...).  Lane l of a slice
// owns row 32k + l and loads that row's segment bounds for this CTA's tile.  Pipeline per
// warp: the row ids of slice k + 3W and the segment bounds of slice k + 2W are loaded, and
// slice k is processed: groups of G lanes take one segment each (lane gl loads 16-byte chunks
// gl, gl + G, ... -- RND rounds, 8 tile-local indices per chunk) and UB segments per group are
// loaded back to back before any shared-memory atomic is issued.  With PF, a lane whose
// segment is longer than RND * G chunks also prefetches its next chunk into L1 with the unit.
template <int MODE, int G, int RND, bool PF, bool BATCH>
__global__ void __launch_bounds__(tiled_threads<MODE, RND>(), 1) ecsr_t_tiled_kernel(const TiledArgs a) {
  constexpr bool HAS_W = weighted_mode(MODE);
  constexpr bool HAS_X = (MODE == kRowVal || MODE == kWRow);
  constexpr unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* acc = reinterpret_cast<uint32_t*>(smem);
  const uint32_t acc_s = (uint32_t)__cvta_generic_to_shared(acc);
  const uint32_t tile_w = (uint32_t)a.tile_w;
  const uint32_t lpad = (tile_w + (uint32_t)(threadIdx.x & 31)) * 0x10001u;  // this lane's dummy word, twice
  const uint4 lane_pads = make_uint4(lpad, lpad, lpad, lpad);
  int* s_boff = reinterpret_cast<int*>(smem + sizeof(uint32_t) * (size_t)a.acc_words);  // kBlockGroup + 1
  __shared__ int s_wsum[32];

  cg::cluster_group cluster = cg::this_cluster();
  const int R = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tile = blockIdx.x / R;
  // vector blockIdx.y of a batch (a separate instantiation: the offsets cost measurable time
  // in the single-vector call)
  const int32_t* __restrict__ lists = BATCH ? a.lists + (int64_t)blockIdx.y * a.nb * kCompactRows : a.lists;
  const int32_t* __restrict__ counts = BATCH ? a.counts + (int64_t)blockIdx.y * a.nb : a.counts;
  const float* __restrict__ row_val = (BATCH && HAS_X) ? a.row_val + (int64_t)blockIdx.y * a.m : a.row_val;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;

  {
    uint4* acc4 = reinterpret_cast<uint4*>(acc);
    for (int i = tid; i < (a.acc_words >> 2); i += nthr) acc4[i] = make_uint4(0u, 0u, 0u, 0u);
  }

  const int b0 = (int)((int64_t)rank * a.nb / R), b1 = (int)((int64_t)(rank + 1) * a.nb / R);
  const int64_t so_stride = a.n_tiles + 1;

  // the compaction kernel of this call may still be running (programmatic dependent launch)
  cudaGridDependencySynchronize();

  // groups of at most one compaction block per thread (nthr <= kBlockGroup)
  for (int g0 = b0; g0 < b1; g0 += nthr) {
    const int ng = min(nthr, b1 - g0);
    __syncthreads();  // s_boff of the previous group is no longer read
    int v = tid < ng ? counts[g0 + tid] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      int t = s_wsum[lane], ti = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int u = __shfl_up_sync(FULL, ti, o);
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

    auto block_of = [&](int g) -> int {
      int lo = 0, hi = ng;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (s_boff[mid] <= g) lo = mid;
        else hi = mid;
      }
      return lo;
    };
    // row id of element 32k + lane of the group's list (-1 past the end); `blk` is the lane's
    // running block hint (the lane's elements only grow)
    auto fetch_row = [&](int k, int& blk) -> int32_t {
      const int g = (k << 5) + lane;
      if (k >= nslices || g >= total) return -1;
      while (s_boff[blk + 1] <= g) ++blk;  // blocks hold ~rate*4096 rows: a step or two
      return __ldg(lists + (int64_t)(g0 + blk) * kCompactRows + (g - s_boff[blk]));
    };
    auto fetch_desc = [&](int32_t row, uint32_t& st, uint32_t& nch, float& xv) {
      st = 0;
      nch = 0;
      xv = 0.0f;
      if (row >= 0) {
        const uint32_t* so = a.seg_off + (int64_t)row * so_stride + tile;
        st = __ldg(so);
        nch = __ldg(so + 1) - st;
        if (HAS_X) xv = __ldg(row_val + row);
      }
    };

    const int gmax = max(total - 1, 0);
    int k = warp;
    int blk = block_of(min((k << 5) + lane, gmax));
    uint32_t cst, cn, nst, nn, mst, mn;
    float cxv, nxv, mxv;
    fetch_desc(fetch_row(k, blk), cst, cn, cxv);                 // slice k
    fetch_desc(fetch_row(k + nwarps, blk), nst, nn, nxv);        // slice k + W
    int32_t row2 = fetch_row(k + 2 * nwarps, blk);               // slice k + 2W

    // A unit is UB rounds of a slice: in round u, lane group grp takes segment grp + u * NG and
    // lane gl loads its chunks gl, gl + G, ... (RND of them), 8 tile-local indices each.
    constexpr int NG = 32 / G;
    constexpr int UBMAX = (HAS_W ? 1 : 2) / RND > 0 ? (HAS_W ? 1 : 2) / RND : 1;
    constexpr int UB = UBMAX > G ? G : UBMAX;
    constexpr int NU = G / UB;  // units per slice
    const int grp = lane / G, gl = lane % G;
    struct Unit {
      uint4 vv[UB][RND];
      float4 w0[UB][RND], w1[UB][RND];
      uint32_t st[UB], ln[UB], lim[UB][RND];
      float xs[UB];
    };
    auto load_unit = [&](Unit& U, uint32_t sst, uint32_t sn, float sxv, int u0) {
#pragma unroll
      for (int u = 0; u < UB; ++u) {
        const int j = grp + (u0 + u) * NG;
        U.st[u] = __shfl_sync(FULL, sst, j);
        U.ln[u] = __shfl_sync(FULL, sn, j);
        U.xs[u] = HAS_X ? __shfl_sync(FULL, sxv, j) : 0.0f;
#pragma unroll
        for (int r = 0; r < RND; ++r) {
          // every lane loads a chunk of its segment (chunk 0, or the chunk where the empty
          // segment would start, past the end); lanes past the end add nothing (lim = 0)
          const uint32_t c = gl + r * G;
          const bool in = c < U.ln[u];
          U.lim[u][r] = in ? tile_w : 0u;
          const uint64_t e = 8ull * (U.st[u] + (in ? c : 0u));
          if (MODE == kFix) {
            // one 48-byte record a chunk (indices, then integer weights): one read a segment;
            // pads and idle lanes add 0 to the spare words
            const uint4* fp = a.fx + 3ull * (U.st[u] + (in ? c : 0u));
            const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            U.vv[u][r] = in ? __ldcs(fp) : lane_pads;
            U.w0[u][r] = in ? __ldcs(reinterpret_cast<const float4*>(fp + 1)) : z;
            U.w1[u][r] = in ? __ldcs(reinterpret_cast<const float4*>(fp + 2)) : z;
          } else if (MODE == kFix24) {
            const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (in) fix24_load(a.fx, U.st[u] + c, U.vv[u][r], U.w0[u][r], U.w1[u][r]);
            else {
              U.vv[u][r] = lane_pads;
              U.w0[u][r] = z;
              U.w1[u][r] = z;
            }
          } else if (MODE == kCount) {
            U.vv[u][r] = in ? ld_stream_u4(a.idx + e) : lane_pads;
          } else {
            U.vv[u][r] = ld_stream_u4(a.idx + e);
          }
          if (HAS_W && !fixed_mode(MODE)) {
            U.w0[u][r] = ld_stream_f4(a.w + e);
            U.w1[u][r] = ld_stream_f4(a.w + e + 4);
          }
        }
        if (PF) {
          // the lane's first chunk past RND * G (segments longer than a unit covers) into L1
          // now, so the extra-chunk loop of consume_unit does not wait on memory
          const uint32_t c = gl + RND * G;
          if (c < U.ln[u]) {
            const uint64_t e = 8ull * (U.st[u] + c);
            prefetch_l1(a.idx + e);
            if (HAS_W) prefetch_l1(a.w + e);
          }
        }
      }
    };
    auto consume_unit = [&](const Unit& U) {
#pragma unroll
      for (int u = 0; u < UB; ++u)
#pragma unroll
        for (int r = 0; r < RND; ++r)
          accumulate8<MODE>(acc_s, U.vv[u][r], HAS_W ? U.w0[u][r] : make_float4(0, 0, 0, 0),
                            HAS_W ? U.w1[u][r] : make_float4(0, 0, 0, 0), U.xs[u], U.lim[u][r]);
      // chunks beyond RND*G (long segments), loaded here
#pragma unroll
      for (int u = 0; u < UB; ++u) {
        for (uint32_t c = gl + RND * G; c < U.ln[u]; c += G) {
          const uint64_t e = 8ull * (U.st[u] + c);
          uint4 x;
          float4 y0 = make_float4(0, 0, 0, 0), y1 = y0;
          if (MODE == kFix) {
            const uint4* fp = a.fx + 3ull * (U.st[u] + c);
            x = __ldcs(fp);
            y0 = __ldcs(reinterpret_cast<const float4*>(fp + 1));
            y1 = __ldcs(reinterpret_cast<const float4*>(fp + 2));
          } else if (MODE == kFix24) {
            fix24_load(a.fx, U.st[u] + c, x, y0, y1);
          } else {
            x = ld_stream_u4(a.idx + e);
            if (HAS_W) {
              y0 = ld_stream_f4(a.w + e);
              y1 = ld_stream_f4(a.w + e + 4);
            }
          }
          accumulate8<MODE>(acc_s, x, y0, y1, U.xs[u], tile_w);
        }
      }
    };
    Unit cur, nxt;
    load_unit(cur, cst, cn, cxv, 0);
    while (k < nslices) {
      fetch_desc(row2, mst, mn, mxv);                            // slice k + 2W
      row2 = fetch_row(k + 3 * nwarps, blk);                     // slice k + 3W
      // This slice's units: the loads of the next unit (of this slice, or the first unit of
      // slice k + W) are issued before the current unit's atomics.
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        if (u + 1 < NU) load_unit(nxt, cst, cn, cxv, (u + 1) * UB);
        else load_unit(nxt, nst, nn, nxv, 0);
        consume_unit(cur);
        cur = nxt;
      }
      cst = nst;
      cn = nn;
      cxv = nxv;
      nst = mst;
      nn = mn;
      nxv = mxv;
      k += nwarps;
    }
  }

  // ---- reduce the cluster's accumulators and write the tile
  cluster.sync();
  const int slice = a.acc_words / R;  // multiple of 4
  const int c0 = rank * slice;
  const float w = (MODE == kCount || MODE == kRowVal) ? __ldg(a.w_homo) : 0.0f;
  const int64_t col_base = (int64_t)tile * a.tile_w;
  float* __restrict__ out = BATCH ? a.out + (int64_t)blockIdx.y * a.n : a.out;
  for (int c = c0 + 4 * tid; c < c0 + slice; c += 4 * nthr) {
    uint4 x[8];
#pragma unroll
    for (int r = 0; r < 8; ++r)
      if (r < R) x[r] = *reinterpret_cast<const uint4*>(cluster.map_shared_rank(acc, r) + c);
    float o[4];
    if (MODE == kCount || fixed_mode(MODE)) {
      uint4 s = make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        if (r < R) {
          s.x += x[r].x;
          s.y += x[r].y;
          s.z += x[r].z;
          s.w += x[r].w;
        }
      }
      if (fixed_mode(MODE)) {  // two's-complement sums; 2^-k is exact
        const float sc = __int_as_float((127 - (int)__ldg(a.meta + 2)) << 23);
        o[0] = __fmul_rn((float)(int32_t)s.x, sc);
        o[1] = __fmul_rn((float)(int32_t)s.y, sc);
        o[2] = __fmul_rn((float)(int32_t)s.z, sc);
        o[3] = __fmul_rn((float)(int32_t)s.w, sc);
      } else {
        o[0] = (float)s.x * w;
        o[1] = (float)s.y * w;
        o[2] = (float)s.z * w;
        o[3] = (float)s.w * w;
      }
    } else {
      float4 s = make_float4(0, 0, 0, 0);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        if (r < R) {
          s.x += __uint_as_float(x[r].x);
          s.y += __uint_as_float(x[r].y);
          s.z += __uint_as_float(x[r].z);
          s.w += __uint_as_float(x[r].w);
        }
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
      *reinterpret_cast<float4*>(out + gc) = make_float4(o[0], o[1], o[2], o[3]);
    } else {
      for (int q = 0; q < 4; ++q)
        if (c + q < a.tile_w && gc + q < a.n) out[gc + q] = o[q];
    }
  }
  cluster.sync();
}

// ---------------------------------------------------------------------------
// split accumulation: counting plans (homogeneous weight, events)
// ---------------------------------------------------------------------------
// DRAM serves random reads of up to ~128 bytes at a fixed rate of row activations, so the
// number of segment reads sets a call's floor.  A counting plan's tiles are up to 65,472
// columns wide (16 tiles at N = 1e6, against the cluster path's ~28K columns), so a call reads
// fewer, longer segments.  CTA (tile t, split q)
// counts the active rows of compaction blocks [q nb / R, (q + 1) nb / R) for its tile and
// writes them to the workspace; split_reduce_kernel adds the R partial counts of a column and
// writes (float)count * w.
//   - Counting: 16-bit counters, two columns a word, one unpredicated shared-memory add per
//     entry (a predicated add costs twice the instructions).  Pad entries land on the 32 pad
//     columns past the tile (the plan spreads its pad values over them); an inactive lane or an
//     empty segment gets a chunk of this lane's pad column, so the lanes of one add
//     instruction rarely meet on a word.  A CTA that could overflow a 16-bit count (a row
//     holding a column twice, or more than 65,535 active rows in its share) counts in 32 bits
//     instead, two passes over its rows, one for each half of the tile.
//   - Work: the CTA tabulates its rows' segments in shared memory (start chunk, chunk prefix)
//     and deals the flattened chunks out in rounds of 32, round r to warp r mod W, chunk
//     32 r + l to lane l; the warps stay within a round of each other whatever the segment
//     lengths, and the loads of the next rounds are in flight while a round's adds issue.
//   - Partial counts are written as the 16-bit pairs, or as 32-bit counts in the 32-bit mode.
constexpr int kFlatRows = 4096;    // rows a CTA-wide pass tabulates
constexpr int kFlatRounds = 1024;  // rounds of 32 chunks a pass holds (32,768 chunks)
constexpr int kSplitMaxSplits = 16;
constexpr int kSplitMaxTile = 65472;  // a multiple of 64; pads reach tile_w + 31 < 65536

// accumulator words: the tile and its 32 pad columns as 16-bit pairs (or, in the 32-bit mode,
// one half of the tile's columns), a multiple of 4
__host__ __device__ inline int split_acc_words(int tile_w) { return ((tile_w + kPlanPadSpan) / 2 + 3) / 4 * 4; }
static size_t split_table_bytes() { return sizeof(uint32_t) * (size_t)(2 * kFlatRows + kFlatRows / 32 + 2 * kFlatRounds); }
static size_t split_smem_bytes(int tile_w, bool tables = true) {
  return sizeof(uint32_t) * (size_t)split_acc_words(tile_w) + sizeof(int) * (kBlockGroup + 1) +
         (tables ? split_table_bytes() : 0);
}

struct SplitArgs {
  const uint32_t* seg_off;
  const uint16_t* idx;
  const uint32_t* meta;
  const int32_t* lists;
  const int32_t* counts;
  uint32_t* part;  // [n_tiles * R][tile_w] words: 16-bit pairs in the first tile_w / 2, or 32-bit counts
  uint32_t* fmt;   // [n_tiles * R]: 0 = 16-bit pairs, 1 = 32-bit counts
  int64_t m, n;
  int32_t tile_w, n_tiles, nb, R;
};

// G == 0: the flat rounds above.  G > 0: warps walk slices of 32 active rows; groups of G lanes
// take one segment each (lane gl loads chunks gl, gl + G, ..., RND in the first round, the
// rest in a loop), and the loads of a slice's next round of segments are in flight while the
// current round's adds issue.  No tables: fewer instructions a chunk than the flat rounds.
template <int G, int RND>
__global__ void __launch_bounds__(kTiledThreads, 1) ecsr_t_split_kernel(const SplitArgs a) {
  constexpr unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  const int acc_words = split_acc_words(a.tile_w);
  const int half_w = a.tile_w >> 1;  // columns of one half of the tile (the 32-bit mode's passes)
  uint32_t* acc = reinterpret_cast<uint32_t*>(smem);
  const uint32_t acc_s = (uint32_t)__cvta_generic_to_shared(acc);
  int* s_boff = reinterpret_cast<int*>(acc + acc_words);  // kBlockGroup + 1
  // pass tables: start chunk and exclusive chunk prefix of each tabulated row, empty-segment
  // bits, and per round the bitmask of segment starts in it and the segment of its first chunk
  uint32_t* t_st = reinterpret_cast<uint32_t*>(s_boff + kBlockGroup + 1);
  uint32_t* t_P = t_st + kFlatRows;
  uint32_t* t_emp = t_P + kFlatRows;
  uint32_t* t_M = t_emp + kFlatRows / 32;
  uint32_t* t_first = t_M + kFlatRounds;
  __shared__ int s_wsum[32];
  __shared__ int s_cut;
  __shared__ uint32_t s_tot;
  const int tile = blockIdx.x / a.R, q = blockIdx.x % a.R;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
  const uint32_t tile_w = (uint32_t)a.tile_w;
  const uint32_t pad2 = (tile_w + (uint32_t)lane) * 0x10001u;
  const uint4 pads = make_uint4(pad2, pad2, pad2, pad2);  // a chunk that adds only to this lane's dummy word
  const int64_t so_stride = a.n_tiles + 1;
  {
    uint4* acc4 = reinterpret_cast<uint4*>(acc);
    for (int i = tid; i < (acc_words >> 2); i += nthr) acc4[i] = make_uint4(0u, 0u, 0u, 0u);
  }
  const int b0 = (int)((int64_t)q * a.nb / a.R), b1 = (int)((int64_t)(q + 1) * a.nb / a.R);

  // the compaction kernel of this call may still be running (programmatic dependent launch)
  cudaGridDependencySynchronize();

  // 16-bit pairs: column x adds 1 to the low (x even) or high (x odd) half of word x / 2; pads
  // land on the pairs past the tile.  32-bit mode: columns [lo, lo + half_w) only.
  uint32_t lo = 0;
  bool wide = false;
  auto add8 = [&](const uint4 v) {
    const uint32_t x[8] = {v.x & 0xFFFFu, v.x >> 16, v.y & 0xFFFFu, v.y >> 16,
                           v.z & 0xFFFFu, v.z >> 16, v.w & 0xFFFFu, v.w >> 16};
    if (!wide) {
#pragma unroll
      for (int e = 0; e < 8; ++e)
        asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(acc_s + ((x[e] >> 1) << 2)), "r"(1u << ((x[e] & 1u) << 4)));
    } else {
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const uint32_t y = x[e] - lo;
        asm volatile("{\n\t.reg .pred p;\n\tsetp.lt.u32 p, %0, %1;\n\t@p red.shared.add.u32 [%2], 1;\n\t}" ::"r"(y),
                     "r"((uint32_t)half_w), "r"(acc_s + (y << 2)));
      }
    }
  };
  // exclusive prefix of the active-row counts of blocks [g0, g0 + ng) into s_boff; returns the total
  auto group_prefix = [&](int g0, int ng) -> int {
    __syncthreads();  // s_boff / s_wsum of an earlier use are no longer read
    int v = tid < ng ? __ldg(a.counts + g0 + tid) : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      int t = lane < nwarps ? s_wsum[lane] : 0, ti = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int u = __shfl_up_sync(FULL, ti, o);
        if (lane >= o) ti += u;
      }
      s_wsum[lane] = ti - t;
    }
    __syncthreads();
    if (tid < ng) s_boff[tid] = s_wsum[warp] + incl - v;
    if (tid == ng - 1) s_boff[ng] = s_wsum[warp] + incl;
    __syncthreads();
    return s_boff[ng];
  };
  auto split_rows = [&]() -> int {
    int my = 0;
    for (int b = b0 + tid; b < b1; b += nthr) my += __ldg(a.counts + b);
    my = warp_sum(my);
    __syncthreads();
    if (lane == 0) s_wsum[warp] = my;
    __syncthreads();
    int t = 0;
    for (int i = 0; i < nwarps; ++i) t += s_wsum[i];
    return t;
  };
  // element j of the group's list of active rows (blocks g0 .. g0 + ng)
  auto row_of = [&](int g0, int ng, int j) -> int32_t {
    int l = 0, h = ng;
    while (h - l > 1) {
      const int mid = (l + h) >> 1;
      if (s_boff[mid] <= j) l = mid;
      else h = mid;
    }
    return __ldg(a.lists + (int64_t)(g0 + l) * kCompactRows + (j - s_boff[l]));
  };

  // slices of 32 active rows per warp, groups of G lanes per segment (G > 0)
  auto run_groups = [&](int g0, int ng, int total) {
    constexpr int GG = G > 0 ? G : 1;
    constexpr int NG = 32 / GG;  // segments a round
    const int grp = lane / GG, gl = lane % GG;
    const int nslices = (total + 31) >> 5;
    auto bounds = [&](int k, uint32_t& st, uint32_t& nch) {
      const int i = (k << 5) + lane;
      st = 0u;
      nch = 0u;
      if (k < nslices && i < total) {
        const uint32_t* so = a.seg_off + (int64_t)row_of(g0, ng, i) * so_stride + tile;
        st = __ldg(so);
        nch = __ldg(so + 1) - st;
      }
    };
    uint32_t st, nch, nst, nnch;
    int k = warp;
    bounds(k, st, nch);
    for (; k < nslices; k += nwarps) {
      bounds(k + nwarps, nst, nnch);  // the warp's next slice, in flight meanwhile
      uint4 cur[RND], nxt[RND];
      uint32_t cst, cn;
      auto load = [&](uint4 (&v)[RND], int u, uint32_t& sst, uint32_t& sn) {
        const int j = u * NG + grp;
        sst = __shfl_sync(FULL, st, j);
        sn = __shfl_sync(FULL, nch, j);
#pragma unroll
        for (int r = 0; r < RND; ++r) {
          const uint32_t c = (uint32_t)(gl + r * GG);
          v[r] = c < sn ? ld_stream_u4(a.idx + 8ull * (sst + c)) : pads;
        }
      };
      load(cur, 0, cst, cn);
#pragma unroll
      for (int u = 0; u < GG; ++u) {
        uint32_t xst = 0u, xn = 0u;
        if (u + 1 < GG) load(nxt, u + 1, xst, xn);
#pragma unroll
        for (int r = 0; r < RND; ++r) add8(cur[r]);
        for (uint32_t c = (uint32_t)(gl + RND * GG); c < cn; c += GG) add8(ld_stream_u4(a.idx + 8ull * (cst + c)));
        if (u + 1 < GG) {
#pragma unroll
          for (int r = 0; r < RND; ++r) cur[r] = nxt[r];
          cst = xst;
          cn = xn;
        }
      }
      st = nst;
      nch = nnch;
    }
  };

  // CTA-wide passes over the `total` active rows of one group: up to kFlatRows rows and
  // kFlatRounds * 32 chunks a pass (a pass stops before a row that would overflow its rounds;
  // a row longer than a whole pass goes through row_loop instead)
  auto run_flat = [&](int g0, int ng, int total) {
    const uint32_t lane_le1 = (lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u)) & ~1u;
    for (int i0 = 0; i0 < total;) {
      const int cnt = min(kFlatRows, total - i0);
      __syncthreads();  // the previous pass's tables are no longer read
      for (int i = tid; i < kFlatRows / 32; i += nthr) t_emp[i] = 0u;
      if (tid == 0) s_cut = cnt;
      __syncthreads();
      {
        uint32_t st[kFlatRows / kTiledThreads], en[kFlatRows / kTiledThreads];
#pragma unroll
        for (int k = 0; k < kFlatRows / kTiledThreads; ++k) {
          const int i = tid + k * nthr;
          st[k] = en[k] = 0u;
          if (i < cnt) {
            const uint32_t* so = a.seg_off + (int64_t)row_of(g0, ng, i0 + i) * so_stride + tile;
            st[k] = __ldg(so);
            en[k] = __ldg(so + 1);
          }
        }
#pragma unroll
        for (int k = 0; k < kFlatRows / kTiledThreads; ++k) {
          const int i = tid + k * nthr;
          if (i < cnt) {
            t_st[i] = st[k];
            t_P[i] = max(en[k] - st[k], 1u);  // an empty segment takes one chunk of pads
            if (en[k] == st[k]) atomicOr(&t_emp[i >> 5], 1u << (i & 31));
          }
        }
      }
      __syncthreads();
      {
        constexpr int PER = kFlatRows / kTiledThreads;  // consecutive rows a thread
        uint32_t c[PER], loc = 0;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
          const int i = PER * tid + k;
          c[k] = i < cnt ? t_P[i] : 0u;
          loc += c[k];
        }
        uint32_t incl = loc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(FULL, incl, o);
          if (lane >= o) incl += t;
        }
        if (lane == 31) s_wsum[warp] = (int)incl;
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
        uint32_t run = (uint32_t)s_wsum[warp] + incl - loc;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
          const int i = PER * tid + k;
          if (i < cnt) {
            t_P[i] = run;
            run += c[k];
            if (run > (uint32_t)(32 * kFlatRounds)) atomicMin(&s_cut, i);  // row i ends past the pass
            if (i == cnt - 1) s_tot = run;
          }
        }
      }
      __syncthreads();
      const int cut = s_cut;
      if (cut == 0) {
        // the pass's first row alone exceeds the tables (only a row holding columns many times
        // can): its chunks go lane by lane, 8 lanes a chunk row
        const uint32_t st = t_st[0], nch = (cut + 1 < cnt ? t_P[1] : s_tot);
        if (!((t_emp[0] >> 0) & 1u))
          for (uint32_t c = tid; c < nch; c += nthr) add8(ld_stream_u4(a.idx + 8ull * (st + c)));
        i0 += 1;
        continue;
      }
      const uint32_t Ctot = cut < cnt ? t_P[cut] : s_tot;
      const int nr = min((int)((Ctot + 31u) >> 5), kFlatRounds);
      for (int r = tid; r < nr; r += nthr) t_M[r] = 0u;
      __syncthreads();
      for (int i = tid; i < cut; i += nthr) {
        const uint32_t p = t_P[i], e = (i + 1 < cut) ? t_P[i + 1] : Ctot;
        atomicOr(&t_M[p >> 5], 1u << (p & 31u));
        for (uint32_t r = (p + 31u) >> 5; (r << 5) < e && r < (uint32_t)nr; ++r) t_first[r] = (uint32_t)i;
      }
      __syncthreads();
      // round r: lane l takes chunk 32 r + l, owned by the segment of the round's first chunk plus
      // the segment starts at positions 1 .. l of the round
      auto round_load = [&](int r) -> uint4 {
        if (r >= nr) return pads;
        const uint32_t g = ((uint32_t)r << 5) + lane;
        if (g >= Ctot) return pads;
        const uint32_t o = min(t_first[r] + __popc(t_M[r] & lane_le1), (uint32_t)cut - 1u);
        if ((t_emp[o >> 5] >> (o & 31u)) & 1u) return pads;
        return ld_stream_u4(a.idx + 8ull * (t_st[o] + (g - t_P[o])));
      };
      int r = warp;
      uint4 v0 = round_load(r), v1 = round_load(r + nwarps);
      for (; r < nr; r += nwarps) {
        const uint4 v2 = round_load(r + 2 * nwarps);
        add8(v0);
        v0 = v1;
        v1 = v2;
      }
      i0 += cut;
    }
  };

  const bool one_group = b1 - b0 <= nthr;
  const int rows = one_group ? (b1 > b0 ? group_prefix(b0, b1 - b0) : 0) : split_rows();
  // 16-bit pairs are exact while no column gets 65,536 adds: no row holds a column twice and
  // the CTA sees at most 65,535 active rows.  Otherwise two passes of 32-bit counts, one for
  // each half of the tile.
  wide = !(__ldg(a.meta) != 0u && rows <= 65535);
  uint32_t* __restrict__ part = a.part + (size_t)blockIdx.x * (size_t)a.tile_w;
  auto run_all = [&]() {
    if (one_group) {
      if constexpr (G > 0) run_groups(b0, b1 - b0, rows);
      else run_flat(b0, b1 - b0, rows);
    } else {
      for (int g0 = b0; g0 < b1; g0 += nthr) {
        const int ng = min(nthr, b1 - g0);
        const int tot = group_prefix(g0, ng);
        if constexpr (G > 0) run_groups(g0, ng, tot);
        else run_flat(g0, ng, tot);
      }
    }
    __syncthreads();
  };
  const uint4* acc4 = reinterpret_cast<const uint4*>(acc);
  if (!wide) {
    run_all();
    uint4* p4 = reinterpret_cast<uint4*>(part);
    for (int i = tid; i < (a.tile_w >> 3); i += nthr) p4[i] = acc4[i];  // tile_w / 2 words of pairs
  } else {
    for (int pass = 0; pass < 2; ++pass) {
      lo = (uint32_t)(pass * half_w);
      run_all();
      uint4* p4 = reinterpret_cast<uint4*>(part + lo);
      for (int i = tid; i < (half_w >> 2); i += nthr) p4[i] = acc4[i];
      if (pass == 0) {
        __syncthreads();
        uint4* z4 = reinterpret_cast<uint4*>(acc);
        for (int i = tid; i < (acc_words >> 2); i += nthr) z4[i] = make_uint4(0u, 0u, 0u, 0u);
      }
    }
  }
  if (tid == 0) a.fmt[blockIdx.x] = wide ? 1u : 0u;
}

// out[t * tile_w + c] = (float)(sum over the R splits of tile t of their count of column c) * w,
// eight columns a thread
__global__ void __launch_bounds__(256) split_reduce_kernel(const uint32_t* __restrict__ part,
                                                           const uint32_t* __restrict__ fmt,
                                                           const float* __restrict__ w_homo, float* __restrict__ out,
                                                           int64_t n, int32_t tile_w, int32_t n_tiles, int32_t R,
                                                           int32_t vec_out) {
  cudaGridDependencySynchronize();  // the partial counts of this call
  const float w = __ldg(w_homo);
  const int gpt = tile_w >> 3;
  const int64_t groups = (int64_t)n_tiles * gpt;
  for (int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < groups;
       gid += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(gid / gpt);
    const int c8 = (int)(gid - (int64_t)t * gpt) << 3;
    const int64_t gc = (int64_t)t * tile_w + c8;
    if (gc >= n) continue;
    uint32_t s[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
    uint32_t wide = 0u;  // bit q: split q of this tile wrote 32-bit counts
    for (int q = 0; q < R; ++q) wide |= (__ldg(fmt + t * R + q) != 0u ? 1u : 0u) << q;
    if (wide == 0u) {
      // every split wrote 16-bit pairs: loads of four splits in flight at a time
#pragma unroll 4
      for (int q = 0; q < R; ++q) {
        const uint4 x = __ldcs(reinterpret_cast<const uint4*>(part + (size_t)(t * R + q) * (size_t)tile_w + (c8 >> 1)));
        s[0] += x.x & 0xFFFFu;
        s[1] += x.x >> 16;
        s[2] += x.y & 0xFFFFu;
        s[3] += x.y >> 16;
        s[4] += x.z & 0xFFFFu;
        s[5] += x.z >> 16;
        s[6] += x.w & 0xFFFFu;
        s[7] += x.w >> 16;
      }
    } else for (int q = 0; q < R; ++q) {
      const int cta = t * R + q;
      const uint32_t* p = part + (size_t)cta * (size_t)tile_w;
      if (((wide >> q) & 1u) == 0u) {
        const uint4 x = __ldcs(reinterpret_cast<const uint4*>(p + (c8 >> 1)));
        s[0] += x.x & 0xFFFFu;
        s[1] += x.x >> 16;
        s[2] += x.y & 0xFFFFu;
        s[3] += x.y >> 16;
        s[4] += x.z & 0xFFFFu;
        s[5] += x.z >> 16;
        s[6] += x.w & 0xFFFFu;
        s[7] += x.w >> 16;
      } else {
        const uint4 x0 = __ldcs(reinterpret_cast<const uint4*>(p + c8));
        const uint4 x1 = __ldcs(reinterpret_cast<const uint4*>(p + c8 + 4));
        s[0] += x0.x;
        s[1] += x0.y;
        s[2] += x0.z;
        s[3] += x0.w;
        s[4] += x1.x;
        s[5] += x1.y;
        s[6] += x1.z;
        s[7] += x1.w;
      }
    }
    float o[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) o[j] = (float)s[j] * w;
    if (vec_out && gc + 7 < n) {
      *reinterpret_cast<float4*>(out + gc) = make_float4(o[0], o[1], o[2], o[3]);
      *reinterpret_cast<float4*>(out + gc + 4) = make_float4(o[4], o[5], o[6], o[7]);
    } else {
      for (int j = 0; j < 8; ++j)
        if (gc + j < n) out[gc + j] = o[j];
    }
  }
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

static size_t tiled_smem_bytes(int acc_words) {
  return sizeof(uint32_t) * (size_t)acc_words + sizeof(int) * (kBlockGroup + 1);
}

// the tile's counters plus kPlanPadSpan dummy words (where unpredicated adds of pad entries
// land), rounded up to a multiple of 4 words per rank
static int acc_words_for(int tile_w, int R) {
  int q = 4 * R;
  return (tile_w + kPlanPadSpan + q - 1) / q * q;
}

// Raises a kernel's dynamic shared-memory limit to the largest size any launch uses (once per
// device and instantiation; every caller sets the same value, so none can lower it).
template <typename K>
static cudaError_t prepare_kernel(K kfn, bool* done) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (done[dev]) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       max_smem_optin() - (int)kStaticSmemReserve);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e == cudaSuccess) done[dev] = true;
  return e;
}

template <int MODE, int G, int RND, bool PF, bool BATCH = false>
static bp_status launch_tiled_g(const TiledArgs& a, int R, cudaStream_t st) {
  auto kfn = ecsr_t_tiled_kernel<MODE, G, RND, PF, BATCH>;
  static bool done[64] = {false};
  BP_CUDA_TRY(prepare_kernel(kfn, done));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(a.n_tiles * R), (unsigned)a.batch, 1);
  cfg.blockDim = dim3(tiled_threads<MODE, RND>(), 1, 1);
  cfg.dynamicSmemBytes = tiled_smem_bytes(a.acc_words);
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

// (lanes per segment, chunk rounds, L1 prefetch of extra chunks): the plan's chosen variant when set
// (bp_csr_plan.variant = G | RND << 8 | PF << 16, e.g. from an autotuning pass), otherwise
// from the mean segment length in 16-byte chunks; BPGPU_TILED=G,RND,PF overrides both.
static void tiled_config(double chunks, bool has_w, int32_t variant, int& G, int& RND, int& PF) {
  // measured on FixedProb rows (uniform columns) at N = 1e6, K = 1000 (3.9 chunks a segment,
  // lengths spread as a multinomial), back-to-back calls:
  //   counts (homogeneous weight): G=2, RND=2 30.7 us at 2 % events, 100.0 at 10 %; G=4, RND=1
  //     34.6 / 127.9; flat distribution 33.0 and G=8 38.0 at 2 %;
  //   per-synapse float weights (index and weight arrays, 48 bytes a chunk): G=4, RND=1
  //     58.9 / 237.7; G=8, RND=1 61.5 / 252.8; G=2, RND=1 64.4 / 269.6; G=2, RND=2 (768
  //     threads) 65.8 / 260.7;
  //   fixed-weight plans (48-byte records) at 2 %: G=4, RND=1 46.7; G=2, RND=2 49.5; G=8,
  //     RND=1 51.7; G=8, RND=2 60.6; G=2, RND=1 61.3; G=1 71.3.
  if (chunks <= 1.25) { G = 1; RND = 1; }
  else if (chunks <= 2.5) { G = 2; RND = 1; }
  else if (chunks <= 5.0) { G = has_w ? 4 : 2; RND = has_w ? 1 : 2; }
  else if (chunks <= 9.0) { G = 8; RND = 1; }
  else { G = 8; RND = 2; }
  // measured: prefetching a lane's first chunk past RND * G into L1 is neutral (30.3 against
  // 31.0 us counts, 59.2 against 59.5 us weights at 2 %); an L2 prefetch of the next slice's
  // segments, tried before it, was 5 % slower
  PF = 0;
  if (variant > 0) {
    G = variant & 0xFF;
    RND = (variant >> 8) & 0xFF;
    PF = (variant >> 16) & 1;
  }
  static int env[3] = {-1, -1, -1};
  if (env[0] < 0) {
    env[0] = 0;
    const char* e = getenv("BPGPU_TILED");
    if (e) sscanf(e, "%d,%d,%d", &env[0], &env[1], &env[2]);
  }
  if (env[0] > 0) {
    G = env[0];
    RND = env[1] > 0 ? env[1] : 1;
    PF = env[2] != 0;
  }
}

template <int MODE>
static bp_status launch_tiled(const TiledArgs& a, int R, double chunks, cudaStream_t st) {
  int G, RND, PF;
  tiled_config(chunks, weighted_mode(MODE), a.variant, G, RND, PF);
  // fixed-weight plans serve one vector a call: no batch instantiation
#define BP_TILED_CASE(g, r)                                                                           \
  if (G == g && RND == r) {                                                                           \
    if (!fixed_mode(MODE) && a.batch > 1)                                                             \
      return launch_tiled_g<MODE, g, r, false, !fixed_mode(MODE)>(a, R, st);                          \
    return PF ? launch_tiled_g<MODE, g, r, true>(a, R, st) : launch_tiled_g<MODE, g, r, false>(a, R, st); \
  }
  BP_TILED_CASE(1, 1)
  BP_TILED_CASE(2, 1)
  BP_TILED_CASE(4, 1)
  BP_TILED_CASE(2, 2)
  BP_TILED_CASE(8, 1)
  BP_TILED_CASE(8, 2)
#undef BP_TILED_CASE
  set_error("tiled event kernel: no variant G=%d RND=%d", G, RND);
  return BP_ENOTSUP;
}

template <int ET>
static bp_status launch_compact_blocked(const void* events, int64_t m, int batch, int32_t* lists, int32_t* counts,
                                        cudaStream_t st) {
  int nb = (int)((m + kCompactRows - 1) / kCompactRows);
  if (batch > 1) compact_blocked_kernel<ET, true><<<dim3(nb, batch), 256, 0, st>>>(events, m, lists, counts);
  else compact_blocked_kernel<ET, false><<<nb, 256, 0, st>>>(events, m, lists, counts);
  return check_launch("compact_blocked_kernel");
}

static bp_status compact_blocked(const void* events, bp_etype et, int64_t m, int batch, int32_t* lists,
                                 int32_t* counts, cudaStream_t st) {
  switch (et) {
    case BP_EV_BOOL: return launch_compact_blocked<BP_EV_BOOL>(events, m, batch, lists, counts, st);
    case BP_EV_F32_POS: return launch_compact_blocked<BP_EV_F32_POS>(events, m, batch, lists, counts, st);
    case BP_EV_F32_NZ: return launch_compact_blocked<BP_EV_F32_NZ>(events, m, batch, lists, counts, st);
  }
  return BP_EINVAL;
}

// ---------------------------------------------------------------------------
// sparse.csrmv, transpose=0, on a plan: y[i] = sum_j A[i, j] x[j].  CTA (tile t, row split s)
// stages x[t * tile_w, (t + 1) * tile_w) in shared memory and walks row i's segment for tile t
// (4 lanes per row, chunks c, c + 4, ...): the dense-vector gathers come from shared memory
// instead of L2.  Partial sums go to part[t][m] (coalesced); csrmv_n_reduce_kernel adds them
// in tile order.
// ---------------------------------------------------------------------------
template <bool HETER>
__global__ void __launch_bounds__(1024) csrmv_n_planned_kernel(const uint32_t* __restrict__ seg_off,
                                                               const uint16_t* __restrict__ idx,
                                                               const float* __restrict__ w, const float* __restrict__ x,
                                                               int64_t m, int64_t n, int32_t tile_w, int32_t n_tiles,
                                                               int32_t splits, float* __restrict__ part) {
  extern __shared__ float xs[];  // tile_w + kPlanPadSpan: the pad indices read zeros
  const int t = blockIdx.x % n_tiles;
  const int sp = blockIdx.x / n_tiles;
  const int64_t col0 = (int64_t)t * tile_w;
  for (int k = threadIdx.x; k < tile_w; k += blockDim.x) xs[k] = col0 + k < n ? __ldg(x + col0 + k) : 0.0f;
  if (threadIdx.x < kPlanPadSpan) xs[tile_w + threadIdx.x] = 0.0f;
  __syncthreads();
  const int64_t r0 = (int64_t)sp * m / splits, r1 = (int64_t)(sp + 1) * m / splits;
  const int64_t so_stride = (int64_t)n_tiles + 1;
  // groups of 4 lanes per row: a segment's chunks are read as one contiguous run; the next
  // row's segment bounds load while the current row is summed
  const int gl = threadIdx.x & 3;
  const int64_t groups = blockDim.x >> 2;
  auto bounds = [&](int64_t row, uint32_t& st, uint32_t& en) {
    st = en = 0;
    if (row < r1) {
      const uint32_t* so = seg_off + row * so_stride + t;
      st = __ldg(so);
      en = __ldg(so + 1);
    }
  };
  uint32_t nst, nen;
  bounds(r0 + (threadIdx.x >> 2), nst, nen);
  for (int64_t rb = r0; rb < r1; rb += groups) {
    const int64_t row = rb + (threadIdx.x >> 2);
    const uint32_t st = nst, en = nen;
    bounds(row + groups, nst, nen);
    float acc = 0.0f;
    for (uint32_t c = st + gl; c < en; c += 4) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(idx + 8ull * c));
      const uint32_t q[8] = {v.x & 0xFFFFu, v.x >> 16, v.y & 0xFFFFu, v.y >> 16,
                             v.z & 0xFFFFu, v.z >> 16, v.w & 0xFFFFu, v.w >> 16};
      if (HETER) {
        const float4 w0 = __ldg(reinterpret_cast<const float4*>(w + 8ull * c));
        const float4 w1 = __ldg(reinterpret_cast<const float4*>(w + 8ull * c + 4));
        const float ww[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
        // pad entries read a zero past the tile with a zero weight: they add +0 (acc starts at +0
        // and a sum of floats is never -0 unless every term is), no test needed
#pragma unroll
        for (int k = 0; k < 8; ++k) acc = fmaf(ww[k], xs[q[k]], acc);
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) acc += xs[q[k]];
      }
    }
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    acc += __shfl_xor_sync(0xffffffffu, acc, 2);
    if (gl == 0 && row < r1) part[(int64_t)t * m + row] = acc;
  }
}

__global__ void __launch_bounds__(256) csrmv_n_reduce_kernel(const float* __restrict__ part, int64_t m,
                                                             int32_t n_tiles, const float* __restrict__ w_homo,
                                                             float* __restrict__ out) {
  const float w = w_homo ? __ldg(w_homo) : 1.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int t = 0; t < n_tiles; ++t) s += __ldg(part + (int64_t)t * m + i);
    out[i] = w_homo ? __fmul_rn(s, w) : s;
  }
}

// how many clusters of R CTAs with `smem` bytes of shared memory can be resident at once
static int max_active_clusters(int R, size_t smem) {
  auto kfn = ecsr_t_tiled_kernel<kCount, 4, 1, true, false>;
  static bool done[64] = {false};
  if (prepare_kernel(kfn, done) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
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

// fills the plan-dependent kernel arguments; checks the tile fits shared memory
static bp_status tiled_args_from_plan(const bp_csr_plan* plan, int cluster, TiledArgs& a, double& chunks,
                                      const char* who) {
  const int acc_words = acc_words_for(plan->tile_w, cluster);
  BP_REQUIRE(tiled_smem_bytes(acc_words) <= (size_t)max_smem_optin() - kStaticSmemReserve, BP_ENOTSUP,
             "%s: tile of %d columns does not fit shared memory", who, plan->tile_w);
  PlanView v = plan_view(plan);
  a = TiledArgs{};
  a.seg_off = v.seg_off;
  a.idx = v.idx;
  a.w = v.w;
  a.meta = v.meta;
  a.batch = 1;
  a.variant = plan->variant;
  a.m = plan->m;
  a.n = plan->n;
  a.tile_w = plan->tile_w;
  a.n_tiles = plan->n_tiles;
  a.nb = (int)((plan->m + kCompactRows - 1) / kCompactRows);
  a.acc_words = acc_words;
  // mean segment length in chunks: entries per (row, tile) plus the average padding
  chunks = ((double)plan->nnz / (double)std::max<int64_t>(plan->m, 1) / (double)plan->n_tiles + 3.5) / 8.0;
  return BP_OK;
}

// Counting plans (kind 1) run the split path: homogeneous weights, single event vectors.
static bool is_split_plan(const bp_csr_plan* plan) { return plan->kind == 1; }

// CTAs per tile of the split path: the tiles share the device's SMs, one CTA each
static int split_count(const bp_csr_plan* plan) {
  const int64_t nb = (plan->m + kCompactRows - 1) / kCompactRows;
  int64_t R = device_sm_count() / std::max<int64_t>(plan->n_tiles, 1);
  R = std::min<int64_t>(R, std::min<int64_t>(nb, kSplitMaxSplits));
  return (int)std::max<int64_t>(R, 1);
}

struct SplitLayout {
  size_t off_counts, off_fmt, off_part, total;
};

static SplitLayout split_layout(const bp_csr_plan* plan) {
  const int64_t nb = (plan->m + kCompactRows - 1) / kCompactRows;
  const int64_t ctas = (int64_t)plan->n_tiles * split_count(plan);
  SplitLayout L;
  L.off_counts = align_up(sizeof(int32_t) * (size_t)nb * kCompactRows, 256);
  L.off_fmt = L.off_counts + align_up(sizeof(int32_t) * (size_t)nb, 256);
  L.off_part = L.off_fmt + align_up(sizeof(uint32_t) * (size_t)ctas, 256);
  L.total = L.off_part + sizeof(uint32_t) * (size_t)ctas * (size_t)plan->tile_w;
  return L;
}

static bp_status split_call(const bp_csr_plan* plan, const float* w_homo, const void* events, bp_etype etype,
                            float* out, void* workspace, cudaStream_t st);

}  // namespace bp

using namespace bp;

extern "C" {

int32_t bp_csr_plan_variants(int32_t* codes, int32_t cap) {
  static const int32_t kVariants[] = {1 | 1 << 8, 2 | 1 << 8, 4 | 1 << 8, 2 | 2 << 8, 8 | 1 << 8, 8 | 2 << 8};
  const int32_t nv = (int32_t)(sizeof(kVariants) / sizeof(kVariants[0]));
  for (int32_t i = 0; codes && i < nv && i < cap; ++i) codes[i] = kVariants[i];
  return nv;
}

int32_t bp_csr_plan_default_tile(int64_t n, int32_t cluster) {
  if (n <= 0) return 0;
  if (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8) cluster = 4;
  const int64_t cap_words =
      ((int64_t)max_smem_optin() - (int64_t)kStaticSmemReserve - 4 * (kBlockGroup + 1)) / 4;
  const int64_t cap_tw = std::min<int64_t>((cap_words - kPlanPadSpan - 32) / 64 * 64, kPlanMaxTileW / 64 * 64);
  // how many clusters of `cluster` CTAs (one CTA per SM) can be resident at once
  int clusters = max_active_clusters(cluster, tiled_smem_bytes(acc_words_for((int)cap_tw, cluster)));
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
  BP_REQUIRE(L.chunks < (1ull << 32), BP_ENOTSUP, "csr_plan_build: %llu padded 16-byte chunks exceed 2^32",
             (unsigned long long)L.chunks);
  BP_REQUIRE(mem != nullptr && bytes >= L.total, BP_ENOMEM, "csr_plan_build: memory %zu < %zu", bytes, L.total);
  BP_REQUIRE((reinterpret_cast<uintptr_t>(mem) & 255u) == 0, BP_EINVAL, "csr_plan_build: memory not 256-byte aligned");
  BP_REQUIRE(m == 0 || (indices && indptr) || nnz == 0, BP_EINVAL, "csr_plan_build: null indices/indptr");
  bp_csr_plan p = {};
  p.m = m;
  p.n = n;
  p.nnz = nnz;
  p.tile_w = tile_w;
  p.n_tiles = (int32_t)nt;
  p.heter = heter ? 1 : 0;
  p.kind = 0;
  p.entries = L.entries;
  p.mem = mem;
  p.bytes = bytes;
  char* base = static_cast<char*>(mem);
  uint32_t* so = reinterpret_cast<uint32_t*>(base + L.off_seg);
  uint16_t* idx = reinterpret_cast<uint16_t*>(base + L.off_idx);
  float* w = heter ? reinterpret_cast<float*>(base + L.off_w) : nullptr;
  uint32_t* meta = reinterpret_cast<uint32_t*>(base + L.off_meta);
  // meta[0] nonzero: no repeated column seen yet; meta[1] = 0: longest row so far (memsets, so
  // that a plan built inside a stream capture stays capturable)
  BP_CUDA_TRY(cudaMemsetAsync(meta, 1, sizeof(uint32_t), st));
  BP_CUDA_TRY(cudaMemsetAsync(meta + 1, 0, sizeof(uint32_t), st));
  if (m > 0) {
    if (nnz == 0) {
      BP_CUDA_TRY(cudaMemsetAsync(so, 0, sizeof(uint32_t) * (size_t)m * (size_t)(nt + 1), st));
    } else {
      int grid = (int)std::min<int64_t>(m, (int64_t)device_sm_count() * 8);
      size_t smem = sizeof(uint32_t) * ((size_t)(3 * nt + 1) + 2 * kPlanDupCheckMax);
      if (smem > 48 * 1024) {
        BP_CUDA_TRY(cudaFuncSetAttribute(plan_build_kernel<int32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
        BP_CUDA_TRY(cudaFuncSetAttribute(plan_build_kernel<int64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
      }
      if (itype == BP_I32)
        plan_build_kernel<int32_t><<<grid, 256, smem, st>>>(static_cast<const int32_t*>(indptr),
                                                             static_cast<const int32_t*>(indices), data, nnz, m, n,
                                                             tile_w, (int)nt, so, idx, w, meta);
      else
        plan_build_kernel<int64_t><<<grid, 256, smem, st>>>(static_cast<const int64_t*>(indptr),
                                                             static_cast<const int64_t*>(indices), data, nnz, m, n,
                                                             tile_w, (int)nt, so, idx, w, meta);
      bp_status s = check_launch("plan_build_kernel");
      if (s != BP_OK) return s;
    }
  }
  *plan_out = p;
  return BP_OK;
}

bp_status bp_csr_plan_arrays(const bp_csr_plan* plan, const uint32_t** seg_off, const uint16_t** idx,
                             const float** w) {
  clear_error();
  BP_REQUIRE(plan != nullptr && plan->mem != nullptr, BP_EINVAL, "csr_plan_arrays: null plan");
  PlanView v = plan_view(plan);
  if (seg_off) *seg_off = v.seg_off;
  if (idx) *idx = v.idx;
  if (w) *w = v.w;
  return BP_OK;
}

size_t bp_event_csrmv_planned_batch_workspace_size(const bp_csr_plan* plan, int32_t batch) {
  if (!plan || plan->m <= 0 || batch <= 0) return 256;
  if (batch == 1 && is_split_plan(plan)) return split_layout(plan).total;
  const int64_t nb = (plan->m + kCompactRows - 1) / kCompactRows;
  return align_up(sizeof(int32_t) * (size_t)batch * (size_t)nb * kCompactRows, 256) +
         align_up(sizeof(int32_t) * (size_t)batch * (size_t)nb, 256);
}

size_t bp_event_csrmv_planned_workspace_size(const bp_csr_plan* plan) {
  return bp_event_csrmv_planned_batch_workspace_size(plan, 1);
}

}  // extern "C"

namespace bp {

// One launch pair for `batch` vectors: vectors (events or dense values) are rows of m, outputs
// rows of n, both contiguous.  `dense` selects sparse.csrmv semantics (vec != 0 rows carry their
// value) over event semantics.
// The entries of a fixed-weight plan whose weights are too small for the fixed point: the rows
// that hold any (rows[0 .. nrows), ascending) and their entries, row i's at [ptr[i], ptr[i + 1])
// of cols / w, added in float by fix_side_kernel after the tiles.
struct FixSide {
  const int32_t* rows;
  const int32_t* ptr;
  const int32_t* cols;
  const float* w;
  int64_t nrows;
  const uint4* fx;  // the plan's chunks as records (bp_csr_plan_fix_interleave)
  int32_t record;   // their size: 48 (int32 weights) or 40 (24-bit weights)
};

// One thread per row with side entries: if the row's event is on, its entries, float atomics
// into out (a few thousand rows at N = 1e6 with N(0.5, 0.1) weights).
template <int ET>
__global__ void __launch_bounds__(256) fix_side_kernel(const void* __restrict__ events, FixSide side, int64_t n,
                                                       float* __restrict__ out) {
  cudaGridDependencySynchronize();  // the tiles of this call have written out
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < side.nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t row = __ldg(side.rows + i);
    bool on;
    if (ET == BP_EV_BOOL) on = __ldg(static_cast<const uint8_t*>(events) + row) != 0;
    else on = ev_on_f32(__ldg(static_cast<const float*>(events) + row), ET);
    if (!on) continue;
    const int32_t e0 = __ldg(side.ptr + i), e1 = __ldg(side.ptr + i + 1);
    for (int32_t e = e0; e < e1; ++e) {
      const int32_t c = __ldg(side.cols + e);
      if ((uint32_t)c < (uint64_t)n) atomicAdd(out + c, __ldg(side.w + e));
    }
  }
}

static bp_status planned_batch(const char* who, const bp_csr_plan* plan, const float* w_homo, const void* vec,
                               bp_etype etype, bool dense, int32_t batch, float* out, int32_t cluster,
                               void* workspace, size_t workspace_bytes, cudaStream_t st,
                               const FixSide* side = nullptr) {
  BP_REQUIRE(plan != nullptr && plan->mem != nullptr, BP_EINVAL, "%s: null plan", who);
  BP_REQUIRE(etype >= BP_EV_BOOL && etype <= BP_EV_F32_NZ, BP_EDTYPE, "%s: bad event type %d", who, (int)etype);
  BP_REQUIRE(batch >= 0 && batch <= 65535, BP_EINVAL, "%s: batch must be in [0, 65535] (got %d)", who, batch);
  if (cluster == 0) cluster = 4;
  BP_REQUIRE(cluster == 1 || cluster == 2 || cluster == 4 || cluster == 8, BP_EINVAL,
             "%s: cluster must be 1, 2, 4 or 8 (got %d)", who, cluster);
  const int64_t m = plan->m, n = plan->n;
  if (n == 0 || batch == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "%s: null out", who);
  if (m == 0 || plan->nnz == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n * (size_t)batch, st));
    return BP_OK;
  }
  BP_REQUIRE(vec != nullptr, BP_EINVAL, "%s: null %s", who, dense ? "vector" : "events");
  const bool homo = plan->heter == 0;
  BP_REQUIRE(!homo || w_homo != nullptr, BP_EINVAL, "%s: homogeneous plan needs w_homo", who);
  const size_t need = bp_event_csrmv_planned_batch_workspace_size(plan, batch);
  BP_REQUIRE(workspace && workspace_bytes >= need, BP_ENOMEM, "%s: workspace %zu < %zu", who, workspace_bytes, need);
  const bool fixed = plan->kind == 2;
  BP_REQUIRE(!fixed || (side != nullptr && plan->heter != 0), BP_EINVAL,
             "%s: a fixed-weight plan runs through bp_event_csrmv_planned_fixed", who);
  BP_REQUIRE(fixed || side == nullptr, BP_EINVAL, "%s: not a fixed-weight plan", who);
  BP_REQUIRE(!fixed || (!dense && batch == 1), BP_ENOTSUP,
             "%s: a fixed-weight plan serves one event vector a call", who);
  if (is_split_plan(plan)) {
    BP_REQUIRE(plan->heter == 0 && plan->tile_w % 64 == 0 && plan->tile_w <= kSplitMaxTile &&
                   split_smem_bytes(plan->tile_w) <= (size_t)max_smem_optin() - kStaticSmemReserve,
               BP_EINVAL, "%s: a counting plan needs a homogeneous weight and a tile of at most %d columns "
               "(bp_csr_plan_count_tile), got %d", who, bp_csr_plan_count_tile(plan->n > 0 ? plan->n : 1), plan->tile_w);
    BP_REQUIRE(!dense && batch == 1, BP_ENOTSUP,
               "%s: a plan of %d-column tiles (16-bit counters) serves one event vector a call; build a plan "
               "with a smaller tile (bp_csr_plan_default_tile) for dense vectors and batches", who, plan->tile_w);
    return split_call(plan, w_homo, vec, etype, out, workspace, st);
  }
  TiledArgs a;
  double chunks = 0.0;
  bp_status s = tiled_args_from_plan(plan, cluster, a, chunks, who);
  if (s != BP_OK) return s;
  int32_t* lists = static_cast<int32_t*>(workspace);
  int32_t* counts = reinterpret_cast<int32_t*>(
      static_cast<char*>(workspace) + align_up(sizeof(int32_t) * (size_t)batch * (size_t)a.nb * kCompactRows, 256));
  ScopedKernelTimer tk(st);  // brackets both kernels of the call
  s = compact_blocked(vec, dense ? BP_EV_F32_NZ : etype, m, batch, lists, counts, st);
  if (s != BP_OK) return s;
  a.lists = lists;
  a.counts = counts;
  a.w_homo = w_homo;
  a.row_val = dense ? static_cast<const float*>(vec) : nullptr;
  a.out = out;
  a.batch = batch;
  a.vec_out = ((reinterpret_cast<uintptr_t>(out) & 15u) == 0 && (batch == 1 || (n & 3) == 0)) ? 1 : 0;
  if (dense) return homo ? launch_tiled<kRowVal>(a, cluster, chunks, st) : launch_tiled<kWRow>(a, cluster, chunks, st);
  if (fixed) {
    a.fx = side->fx;
    s = side->record == 40 ? launch_tiled<kFix24>(a, cluster, chunks, st) : launch_tiled<kFix>(a, cluster, chunks, st);
    if (s != BP_OK || side->nrows == 0) return s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((side->nrows + 255) / 256, device_sm_count() * 8));
    cfg.gridDim = dim3((unsigned)blocks, 1, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    switch (etype) {
      case BP_EV_BOOL: BP_CUDA_TRY(cudaLaunchKernelEx(&cfg, fix_side_kernel<BP_EV_BOOL>, vec, *side, (int64_t)n, out)); break;
      case BP_EV_F32_POS:
        BP_CUDA_TRY(cudaLaunchKernelEx(&cfg, fix_side_kernel<BP_EV_F32_POS>, vec, *side, (int64_t)n, out));
        break;
      default: BP_CUDA_TRY(cudaLaunchKernelEx(&cfg, fix_side_kernel<BP_EV_F32_NZ>, vec, *side, (int64_t)n, out));
    }
    return check_launch("fix_side_kernel");
  }
  return homo ? launch_tiled<kCount>(a, cluster, chunks, st) : launch_tiled<kWeight>(a, cluster, chunks, st);
}

// Converts a heterogeneous plan's float weights to int32 fixed point, q = rint(w * 2^k), in place
// (convert != 0), and lists the nonzero weights with |w| < tau, which the fixed point cannot carry
// within the accuracy bar, as (row, column, w) at side[0 .. count) (up to cap of them; the count
// is always complete).  One warp per row.
__global__ void __launch_bounds__(256) fix_weights_kernel(const uint32_t* __restrict__ seg_off,
                                                          const uint16_t* __restrict__ idx, float* w, int64_t m,
                                                          int tile_w, int n_tiles, float scale_up, float tau,
                                                          int32_t* side_rows, int32_t* side_cols, float* side_w,
                                                          int64_t cap, unsigned long long* count, int convert) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < m; r += nwarps) {
    const uint32_t* so = seg_off + r * (int64_t)(n_tiles + 1);
    for (int t = 0; t < n_tiles; ++t) {
      const uint64_t e0 = 8ull * so[t], e1 = 8ull * so[t + 1];
      for (uint64_t e = e0 + lane; e < e1; e += 32) {
        const uint32_t x = idx[e];
        if (x >= (uint32_t)tile_w) continue;  // padding: weight 0 stays 0
        const float v = w[e];
        const bool small = v != 0.0f && fabsf(v) < tau;
        if (small) {
          const unsigned long long pos = atomicAdd(count, 1ull);
          if ((int64_t)pos < cap) {
            side_rows[pos] = (int32_t)r;
            side_cols[pos] = (int32_t)((int64_t)t * tile_w + x);
            side_w[pos] = v;
          }
        }
        if (convert) w[e] = __int_as_float(small ? 0 : __float2int_rn(v * scale_up));
      }
    }
  }
}

__global__ void set_word_kernel(uint32_t* p, uint32_t v) { *p = v; }

// chunk c of a plan -> fx[3c] = its 8 indices, fx[3c + 1 .. 3c + 2] = its 8 (integer) weights
__global__ void __launch_bounds__(256) fix_interleave_kernel(const uint4* __restrict__ idx,
                                                             const uint4* __restrict__ w, uint4* __restrict__ fx,
                                                             uint64_t nchunks) {
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nchunks;
       c += (uint64_t)gridDim.x * blockDim.x) {
    fx[3 * c] = idx[c];
    fx[3 * c + 1] = w[2 * c];
    fx[3 * c + 2] = w[2 * c + 1];
  }
}

// chunk c of a plan -> its 40-byte record at byte 40c (the layout fix24_load reads): indices,
// low 16 bits of the weights, high bytes (the high bytes first in an odd chunk).  One warp per
// row walks the row's segments, chunks [seg_off[r][0], seg_off[r][T]): the gaps the plan leaves
// between rows hold no entries and are not written.  Weights outside [-2^23, 2^23) are counted
// into *unfit (their records would be wrong).
__global__ void __launch_bounds__(256) fix_interleave24_kernel(const uint32_t* __restrict__ seg_off,
                                                               const uint4* __restrict__ idx,
                                                               const int4* __restrict__ w,
                                                               unsigned char* __restrict__ fx, int64_t m,
                                                               int n_tiles, unsigned long long* unfit) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < m; r += nwarps) {
    const uint32_t* so = seg_off + r * (int64_t)(n_tiles + 1);
    const uint64_t c1 = so[n_tiles];
    for (uint64_t c = so[0] + lane; c < c1; c += 32) {
      const int4 a = w[2 * c], b = w[2 * c + 1];
      const int32_t q[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
      uint32_t lo[4] = {0u, 0u, 0u, 0u}, hi[2] = {0u, 0u};
      int bad = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        bad += (q[j] < -(1 << 23) || q[j] >= (1 << 23)) ? 1 : 0;
        const uint32_t u = (uint32_t)q[j];
        lo[j >> 1] |= (u & 0xFFFFu) << (16 * (j & 1));
        hi[j >> 2] |= ((u >> 16) & 0xFFu) << (8 * (j & 3));
      }
      if (bad) atomicAdd(unfit, (unsigned long long)bad);
      const uint4 x = idx[c];
      uint2* rec = reinterpret_cast<uint2*>(fx + 40ull * c);  // 8-byte aligned
      const uint2 h = make_uint2(hi[0], hi[1]);
      const int o = (int)(c & 1u);  // odd: the high bytes first
      if (o) rec[0] = h;
      rec[o + 0] = make_uint2(x.x, x.y);
      rec[o + 1] = make_uint2(x.z, x.w);
      rec[o + 2] = make_uint2(lo[0], lo[1]);
      rec[o + 3] = make_uint2(lo[2], lo[3]);
      if (!o) rec[4] = h;
    }
  }
}

}  // namespace bp

namespace bp {

// Main-loop form of the split kernel: (G, RND) = (0, 1) for the flat rounds, otherwise G lanes
// a segment and RND chunks a lane in the first round; BPGPU_SPLIT=G,RND overrides the default.
// Measured at N = 1e6, K = 1000, 2 % (segments of ~62 entries): (4, 2) 31.5 us a call, (4, 3)
// 31.5, (2, 4) 32.5, flat 32.9, (8, 1) 34.8, (8, 2) 35.3.
static void split_variant(int& G, int& RND) {
  G = 4;
  RND = 2;
  const char* e = getenv("BPGPU_SPLIT");
  if (e) {
    int g = 0, r = 0;
    if (sscanf(e, "%d,%d", &g, &r) == 2) {
      G = g;
      RND = r;
    }
  }
}

static bp_status split_call(const bp_csr_plan* plan, const float* w_homo, const void* events, bp_etype etype,
                            float* out, void* workspace, cudaStream_t st) {
  PlanView v = plan_view(plan);
  const SplitLayout L = split_layout(plan);
  char* ws = static_cast<char*>(workspace);
  SplitArgs a;
  a.seg_off = v.seg_off;
  a.idx = v.idx;
  a.meta = v.meta;
  a.lists = reinterpret_cast<const int32_t*>(ws);
  a.counts = reinterpret_cast<const int32_t*>(ws + L.off_counts);
  a.fmt = reinterpret_cast<uint32_t*>(ws + L.off_fmt);
  a.part = reinterpret_cast<uint32_t*>(ws + L.off_part);
  a.m = plan->m;
  a.n = plan->n;
  a.tile_w = plan->tile_w;
  a.n_tiles = plan->n_tiles;
  a.nb = (int)((plan->m + kCompactRows - 1) / kCompactRows);
  a.R = split_count(plan);
  ScopedKernelTimer tk(st);  // brackets the call's three kernels
  bp_status s = compact_blocked(events, etype, plan->m, 1, reinterpret_cast<int32_t*>(ws),
                                reinterpret_cast<int32_t*>(ws + L.off_counts), st);
  if (s != BP_OK) return s;
  int sg = 0, srnd = 1;
  split_variant(sg, srnd);
  void (*kfn)(const SplitArgs) = ecsr_t_split_kernel<0, 1>;
  if (sg == 2 && srnd == 4) kfn = ecsr_t_split_kernel<2, 4>;
  else if (sg == 4 && srnd == 2) kfn = ecsr_t_split_kernel<4, 2>;
  else if (sg == 4 && srnd == 3) kfn = ecsr_t_split_kernel<4, 3>;
  else if (sg == 8 && srnd == 1) kfn = ecsr_t_split_kernel<8, 1>;
  else if (sg == 8 && srnd == 2) kfn = ecsr_t_split_kernel<8, 2>;
  else sg = 0;
  static bool done[8][64] = {};
  BP_CUDA_TRY(prepare_kernel(kfn, done[(sg == 0 ? 0 : sg == 2 ? 1 : sg == 4 ? 2 + (srnd == 3) : 4 + (srnd == 2))]));
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(a.n_tiles * a.R), 1, 1);
  cfg.blockDim = dim3(kTiledThreads, 1, 1);
  cfg.dynamicSmemBytes = split_smem_bytes(a.tile_w, sg == 0);
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BP_CUDA_TRY(cudaLaunchKernelEx(&cfg, kfn, a));
  const int64_t groups = (int64_t)a.n_tiles * (a.tile_w >> 3);
  cudaLaunchConfig_t rcfg = {};
  rcfg.gridDim = dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>((groups + 255) / 256, (int64_t)device_sm_count() * 8)), 1, 1);
  rcfg.blockDim = dim3(256, 1, 1);
  rcfg.stream = st;
  rcfg.attrs = attr;
  rcfg.numAttrs = 1;
  const int32_t vec_out = (reinterpret_cast<uintptr_t>(out) & 15u) == 0 ? 1 : 0;
  BP_CUDA_TRY(cudaLaunchKernelEx(&rcfg, split_reduce_kernel, (const uint32_t*)a.part, (const uint32_t*)a.fmt, w_homo,
                                 out, (int64_t)a.n, (int32_t)a.tile_w, (int32_t)a.n_tiles, (int32_t)a.R, vec_out));
  return BP_OK;
}

}  // namespace bp

extern "C" {

int32_t bp_csr_plan_count_tile(int64_t n) {
  // worth it from 2^19 columns: the fewest tiles of at most kSplitMaxTile columns, in multiples
  // of 64, whose 16-bit accumulator and pass tables fit one CTA
  if (n < (1 << 19)) return 0;
  const int64_t nt = (n + kSplitMaxTile - 1) / kSplitMaxTile;
  int64_t tw = (n + nt - 1) / nt;
  tw = (tw + 63) / 64 * 64;
  if (tw > kSplitMaxTile) tw = kSplitMaxTile;
  if (split_smem_bytes((int)tw) > (size_t)max_smem_optin() - kStaticSmemReserve) return 0;
  return (int32_t)tw;
}

}  // extern "C"

extern "C" {

bp_status bp_csr_plan_fix_weights(bp_csr_plan* plan, int32_t k, float tau, int32_t* side_rows, int32_t* side_cols,
                                  float* side_w, int64_t side_cap, uint64_t* side_count, int32_t convert,
                                  bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(plan != nullptr && plan->mem != nullptr, BP_EINVAL, "csr_plan_fix_weights: null plan");
  BP_REQUIRE(plan->heter != 0 && plan->kind == 0, BP_EINVAL,
             "csr_plan_fix_weights: needs a general heterogeneous plan (heter=%d, kind=%d)", plan->heter, plan->kind);
  BP_REQUIRE(k >= 0 && k <= 100, BP_EINVAL, "csr_plan_fix_weights: exponent %d outside [0, 100]", k);
  BP_REQUIRE(side_count != nullptr, BP_EINVAL, "csr_plan_fix_weights: null side count");
  BP_REQUIRE(side_cap <= 0 || (side_rows && side_cols && side_w), BP_EINVAL, "csr_plan_fix_weights: null side arrays");
  PlanView v = plan_view(plan);
  BP_CUDA_TRY(cudaMemsetAsync(side_count, 0, sizeof(uint64_t), st));
  if (plan->m > 0) {
    const int64_t g = std::min<int64_t>((plan->m + 7) / 8, (int64_t)device_sm_count() * 16);
    fix_weights_kernel<<<(unsigned)g, 256, 0, st>>>(v.seg_off, v.idx, const_cast<float*>(v.w), plan->m, plan->tile_w,
                                                  plan->n_tiles, ldexpf(1.0f, k), tau, side_rows, side_cols, side_w,
                                                  side_cap, reinterpret_cast<unsigned long long*>(side_count),
                                                  convert);
    bp_status s = check_launch("fix_weights_kernel");
    if (s != BP_OK) return s;
  }
  if (convert) {
    set_word_kernel<<<1, 1, 0, st>>>(const_cast<uint32_t*>(v.meta) + 2, (uint32_t)k);
    bp_status s = check_launch("set_word_kernel");
    if (s != BP_OK) return s;
    plan->kind = 2;
  }
  return BP_OK;
}

size_t bp_csr_plan_fix_interleave_bytes(const bp_csr_plan* plan, int32_t record_bytes) {
  if (!plan || (record_bytes != 48 && record_bytes != 40)) return 0;
  return (size_t)(plan->entries / 8) * (size_t)record_bytes;
}

bp_status bp_csr_plan_fix_interleave(const bp_csr_plan* plan, int32_t record_bytes, void* fx, size_t fx_bytes,
                                     uint64_t* unfit, bp_stream_t stream) {
  clear_error();
  BP_REQUIRE(plan != nullptr && plan->mem != nullptr && plan->kind == 2, BP_EINVAL,
             "csr_plan_fix_interleave: needs a fixed-weight plan");
  BP_REQUIRE(record_bytes == 48 || (record_bytes == 40 && unfit != nullptr), BP_EINVAL,
             "csr_plan_fix_interleave: records of 48 bytes, or of 40 with an unfit counter (got %d%s)", record_bytes,
             unfit ? "" : ", no counter");
  const size_t need = bp_csr_plan_fix_interleave_bytes(plan, record_bytes);
  BP_REQUIRE(fx != nullptr && fx_bytes >= need && (reinterpret_cast<uintptr_t>(fx) & 15u) == 0, BP_EINVAL,
             "csr_plan_fix_interleave: %zu bytes at %p, need %zu on a 16-byte boundary", fx_bytes, fx, need);
  PlanView v = plan_view(plan);
  const uint64_t nchunks = plan->entries / 8;
  if (nchunks == 0) return BP_OK;
  const uint64_t g = std::min<uint64_t>((nchunks + 255) / 256, (uint64_t)device_sm_count() * 32);
  if (record_bytes == 40) {
    if (plan->m <= 0) return BP_OK;
    const int64_t gr = std::min<int64_t>((plan->m + 7) / 8, (int64_t)device_sm_count() * 16);
    fix_interleave24_kernel<<<(unsigned)gr, 256, 0, as_cuda(stream)>>>(
        v.seg_off, reinterpret_cast<const uint4*>(v.idx), reinterpret_cast<const int4*>(v.w),
        static_cast<unsigned char*>(fx), plan->m, plan->n_tiles, reinterpret_cast<unsigned long long*>(unfit));
    return check_launch("fix_interleave24_kernel");
  }
  fix_interleave_kernel<<<(unsigned)g, 256, 0, as_cuda(stream)>>>(reinterpret_cast<const uint4*>(v.idx),
                                                                 reinterpret_cast<const uint4*>(v.w),
                                                                 static_cast<uint4*>(fx), nchunks);
  return check_launch("fix_interleave_kernel");
}

bp_status bp_event_csrmv_planned_fixed(const bp_csr_plan* plan, const void* fx, int32_t record_bytes,
                                       const int32_t* side_rows,
                                       const int32_t* side_ptr, const int32_t* side_cols, const float* side_w,
                                       int64_t side_nrows, const void* events, bp_etype etype, float* out,
                                       int32_t cluster, void* workspace, size_t workspace_bytes,
                                       bp_stream_t stream) {
  clear_error();
  BP_REQUIRE(side_nrows >= 0 && (side_nrows == 0 || (side_rows && side_ptr && side_cols && side_w)), BP_EINVAL,
             "event_csrmv_planned_fixed: null side arrays for %lld rows", (long long)side_nrows);
  BP_REQUIRE(fx != nullptr && (reinterpret_cast<uintptr_t>(fx) & 15u) == 0, BP_EINVAL,
             "event_csrmv_planned_fixed: the interleaved chunks (bp_csr_plan_fix_interleave) are required");
  BP_REQUIRE(record_bytes == 48 || record_bytes == 40, BP_EINVAL,
             "event_csrmv_planned_fixed: records of 48 or 40 bytes (got %d)", record_bytes);
  FixSide side{side_rows, side_ptr, side_cols, side_w, side_nrows, static_cast<const uint4*>(fx), record_bytes};
  return planned_batch("event_csrmv_planned_fixed", plan, nullptr, events, etype, false, 1, out, cluster, workspace,
                       workspace_bytes, as_cuda(stream), &side);
}

bp_status bp_event_csrmv_planned(const bp_csr_plan* plan, const float* w_homo, const void* events, bp_etype etype,
                                 float* out, int32_t cluster, void* workspace, size_t workspace_bytes,
                                 bp_stream_t stream) {
  clear_error();
  return planned_batch("event_csrmv_planned", plan, w_homo, events, etype, false, 1, out, cluster, workspace,
                       workspace_bytes, as_cuda(stream));
}

bp_status bp_event_csrmv_planned_batch(const bp_csr_plan* plan, const float* w_homo, const void* events,
                                       bp_etype etype, int32_t batch, float* out, int32_t cluster, void* workspace,
                                       size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  return planned_batch("event_csrmv_planned_batch", plan, w_homo, events, etype, false, batch, out, cluster,
                       workspace, workspace_bytes, as_cuda(stream));
}

// sparse.csrmv, transpose=1, on a plan: out[j] = sum_i A[i, j] * vec[i].  Rows with vec[i] == 0
// contribute nothing and are skipped by the compaction (the dense vector is treated as
// events under the != 0 rule); the others carry their value into the tile accumulation.
bp_status bp_csrmv_planned(const bp_csr_plan* plan, const float* w_homo, const float* vec, float* out,
                           int32_t cluster, void* workspace, size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  return planned_batch("csrmv_planned", plan, w_homo, vec, BP_EV_F32_NZ, true, 1, out, cluster, workspace,
                       workspace_bytes, as_cuda(stream));
}

size_t bp_csrmv_planned_n_workspace_size(const bp_csr_plan* plan) {
  if (!plan || plan->m <= 0 || plan->n_tiles <= 0) return 256;
  return align_up(sizeof(float) * (size_t)plan->m * (size_t)plan->n_tiles, 256);
}

bp_status bp_csrmv_planned_n(const bp_csr_plan* plan, const float* w_homo, const float* vec, float* out,
                             void* workspace, size_t workspace_bytes, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(plan != nullptr && plan->mem != nullptr, BP_EINVAL, "csrmv_planned_n: null plan");
  BP_REQUIRE(plan->kind == 0, BP_EINVAL, "csrmv_planned_n: needs a general plan (kind %d)", plan->kind);
  const int64_t m = plan->m, n = plan->n;
  if (m == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "csrmv_planned_n: null out");
  if (n == 0 || plan->nnz == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)m, st));
    return BP_OK;
  }
  BP_REQUIRE(vec != nullptr, BP_EINVAL, "csrmv_planned_n: null vector");
  const bool homo = plan->heter == 0;
  BP_REQUIRE(!homo || w_homo != nullptr, BP_EINVAL, "csrmv_planned_n: homogeneous plan needs w_homo");
  const size_t need = bp_csrmv_planned_n_workspace_size(plan);
  BP_REQUIRE(workspace && workspace_bytes >= need, BP_ENOMEM, "csrmv_planned_n: workspace %zu < %zu", workspace_bytes,
             need);
  const size_t smem = sizeof(float) * ((size_t)plan->tile_w + kPlanPadSpan);
  BP_REQUIRE(smem <= (size_t)max_smem_optin() - kStaticSmemReserve, BP_ENOTSUP,
             "csrmv_planned_n: tile of %d columns does not fit shared memory", plan->tile_w);
  PlanView v = plan_view(plan);
  const int nt = plan->n_tiles;
  float* part = static_cast<float*>(workspace);
  static bool configured[2][64] = {{false}};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  auto kfn = homo ? csrmv_n_planned_kernel<false> : csrmv_n_planned_kernel<true>;
  if (!configured[homo ? 0 : 1][dev]) {
    BP_CUDA_TRY(
        cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_optin() - (int)kStaticSmemReserve));
    configured[homo ? 0 : 1][dev] = true;
  }
  // row splits: as many CTAs as are resident at once (one wave), at least one per tile.  Every
  // CTA walks the same number of rows, so a second partial wave would double the time.
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, 1024, smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  int splits = (int)(((int64_t)per_sm * device_sm_count()) / nt);
  if (splits < 1) splits = 1;
  if ((int64_t)splits > m) splits = (int)m;
  ScopedKernelTimer tk(st);
  kfn<<<nt * splits, 1024, smem, st>>>(v.seg_off, v.idx, homo ? nullptr : v.w, vec, m, n, plan->tile_w, nt, splits,
                                       part);
  bp_status s = check_launch("csrmv_n_planned_kernel");
  if (s != BP_OK) return s;
  int64_t g = (m + 255) / 256;
  const int64_t maxb = (int64_t)device_sm_count() * 16;
  if (g > maxb) g = maxb;
  csrmv_n_reduce_kernel<<<(unsigned)g, 256, 0, st>>>(part, m, nt, homo ? w_homo : nullptr, out);
  return check_launch("csrmv_n_reduce_kernel");
}

bp_status bp_csrmv_planned_batch(const bp_csr_plan* plan, const float* w_homo, const float* vec, int32_t batch,
                                 float* out, int32_t cluster, void* workspace, size_t workspace_bytes,
                                 bp_stream_t stream) {
  clear_error();
  return planned_batch("csrmv_planned_batch", plan, w_homo, vec, BP_EV_F32_NZ, true, batch, out, cluster,
                       workspace, workspace_bytes, as_cuda(stream));
}

}  // extern "C"
