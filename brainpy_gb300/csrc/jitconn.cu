// jitconn.cu -- just-in-time connectivity operators:
//   jitconn.event_mv_prob_{homo,uniform,normal} and jitconn.mv_prob_{homo,uniform,normal}.
//
// y = M v where M is never stored: its connections are regenerated from LFSR88 streams on
// every call, reproducing the reference's Taichi algorithms bit for bit.
//
// Taichi GPU algorithm (brainpy/_src/math/jitconn/_event_matvec_taichi.py:96-155,
// _matvec_taichi.py:79-137): an "owner" (output row when outdim_parallel, input column
// otherwise) has 32 lane streams; lane l is seeded seed + owner*32 + l and walks the stripe
// (step*l - 1 + inc, ..., < min(step*(l+1) - 1, limit)) of the other dimension with
// increments randint(1, clen), step = max((num_row + 1) >> 5, 1), all in uint32.
//   pull (outdim_parallel=1): one warp per output row, lane sums reduced in the warp;
//   push (outdim_parallel=0): one warp per input column (skipped when it carries no event),
//     atomic adds into the output.
// Taichi CPU algorithm (_event_matvec_taichi.py:38-85): one stream per owner seeded
// seed + owner covering the whole other dimension, first index randint(0, clen - 1);
// here one thread per owner.
#include "common.cuh"
#include "lfsr88.cuh"
#include "timer.cuh"

namespace bp {

enum { JC_HOMO = 0, JC_UNIFORM = 1, JC_NORMAL = 2 };
enum { VEC_EV_BOOL = 0, VEC_EV_F32 = 1, VEC_DENSE = 2 };

struct JcArgs {
  const void* vec;
  float* out;
  int64_t num_row, num_col;
  float p0, p1;
  FastMod fm;
  uint32_t seed, step;
};

template <int KIND>
__device__ __forceinline__ float jc_draw(Lfsr88& k, float p0, float p1) {
  if (KIND == JC_UNIFORM) return lfsr88_uniform(k, p0, p1);
  if (KIND == JC_NORMAL) return lfsr88_normal(k, p0, p1);
  return p0;
}

// ---------------------------------------------------------------------------
// Taichi GPU algorithm, pull: warp per output row
// ---------------------------------------------------------------------------
template <int KIND, int VK>
__global__ void __launch_bounds__(256) jc_pull_gpu_kernel(JcArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const uint32_t lim = (uint32_t)a.num_col;
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < a.num_row; row += nwarps) {
    const uint32_t i = (uint32_t)(row * 32 + lane);
    uint32_t c = a.step * (uint32_t)lane - 1u;
    uint32_t end = c + a.step;
    if (lim < end) end = lim;
    Lfsr88 key = lfsr88_key(a.seed + i);
    c += lfsr88_inc(key, a.fm);
    float r = 0.0f;
    while (c < end) {
      const float w = jc_draw<KIND>(key, a.p0, a.p1);
      if (VK == VEC_EV_BOOL) {
        r = __fadd_rn(r, __fmul_rn(w, static_cast<const uint8_t*>(a.vec)[c] ? 1.0f : 0.0f));  // r += w * events[c]
      } else if (VK == VEC_EV_F32) {
        r = __fadd_rn(r, __fmul_rn(w, __ldg(static_cast<const float*>(a.vec) + c)));
      } else {
        const float v = __ldg(static_cast<const float*>(a.vec) + c);
        if (KIND == JC_HOMO) r = __fadd_rn(r, v);  // weight applied once per lane below
        else r = __fadd_rn(r, __fmul_rn(v, w));
      }
      c += lfsr88_inc(key, a.fm);
    }
    if (VK == VEC_DENSE && KIND == JC_HOMO) r = __fmul_rn(a.p0, r);
    r = warp_sum(r);
    if (lane == 0) a.out[row] = r;
  }
}

// ---------------------------------------------------------------------------
// Taichi GPU algorithm, pull, homogeneous weight and bool events: lane-major.
// Stream (row, l) of the algorithm above only visits columns [l * step, (l + 1) * step), so a
// block that takes one lane index l (blockIdx.y) for a run of rows holds the event bits of
// that range in shared memory (step / 8 bytes) and every thread walks one (row, l) stream
// against it: no global gather per generated connection.  The homogeneous weight draws
// nothing from the stream, so a stream contributes (number of active events it visits) * w;
// the counts are added per row as exact integers (into `out`, reinterpreted) and turned into
// count * w by jc_counts_to_out_kernel.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) jc_pull_homo_bool_lanes_kernel(JcArgs a, int64_t rows_per_block) {
  extern __shared__ uint32_t ev_bits[];
  const uint32_t l = blockIdx.y;
  const uint32_t lim = (uint32_t)a.num_col;
  const uint32_t c0 = a.step * l;
  const uint32_t c1 = c0 >= lim ? c0 : (lim - c0 < a.step ? lim : c0 + a.step);
  const uint32_t nwords = (c1 - c0 + 31u) >> 5;
  const uint8_t* ev = static_cast<const uint8_t*>(a.vec);
  for (uint32_t w = threadIdx.x; w < nwords; w += blockDim.x) {
    uint32_t word = 0;
    const uint32_t cb = c0 + 32u * w;
#pragma unroll 8
    for (uint32_t b = 0; b < 32u; ++b)
      if (cb + b < c1 && ev[cb + b]) word |= 1u << b;
    ev_bits[w] = word;
  }
  __syncthreads();
  int32_t* counts = reinterpret_cast<int32_t*>(a.out);
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
  const int64_t r1 = r0 + rows_per_block < a.num_row ? r0 + rows_per_block : a.num_row;
  for (int64_t row = r0 + threadIdx.x; row < r1; row += blockDim.x) {
    const uint32_t i = (uint32_t)(row * 32 + l);
    uint32_t c = c0 - 1u;
    uint32_t end = c + a.step;
    if (lim < end) end = lim;
    Lfsr88 key = lfsr88_key(a.seed + i);
    c += lfsr88_inc(key, a.fm);
    int cnt = 0;
    while (c < end) {  // c0 <= c < c1 here
      const uint32_t o = c - c0;
      cnt += (int)((ev_bits[o >> 5] >> (o & 31u)) & 1u);
      c += lfsr88_inc(key, a.fm);
    }
    if (cnt) atomicAdd(counts + row, cnt);
  }
}

__global__ void __launch_bounds__(256) jc_counts_to_out_kernel(float* __restrict__ out, int64_t n, float w) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = __fmul_rn((float)reinterpret_cast<const int32_t*>(out)[k], w);
}

// ---------------------------------------------------------------------------
// Taichi GPU algorithm, push: warp per input column.  Event vectors: each warp examines 32
// columns at a time (one event per lane, a ballot), then pushes the active ones one after
// another with all 32 lanes; with sparse events the scan is a load per 32 columns instead of a
// dependent load per column.  Homogeneous weights add equal values, so the order of the
// atomic adds does not change the sums.
// ---------------------------------------------------------------------------
template <int KIND, int VK>
__global__ void __launch_bounds__(256) jc_push_gpu_kernel(JcArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t gwarp = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint32_t lim = (uint32_t)a.num_row;
  auto push_column = [&](int64_t col, float cv) {
    const uint32_t i = (uint32_t)(col * 32 + lane);
    uint32_t r = a.step * (uint32_t)lane - 1u;
    uint32_t end = r + a.step;
    if (lim < end) end = lim;
    Lfsr88 key = lfsr88_key(a.seed + i);
    r += lfsr88_inc(key, a.fm);
    while (r < end) {
      const float w = jc_draw<KIND>(key, a.p0, a.p1);
      float add;
      if (VK == VEC_DENSE) add = (KIND == JC_HOMO) ? __fmul_rn(a.p0, cv) : __fmul_rn(w, cv);
      else add = w;  // event push kernels add the weight itself (_event_matvec_taichi.py:121, :250)
      atomicAdd(a.out + r, add);
      r += lfsr88_inc(key, a.fm);
    }
  };
  if (VK == VEC_DENSE) {
    for (int64_t col = gwarp; col < a.num_col; col += nwarps) push_column(col, __ldg(static_cast<const float*>(a.vec) + col));
    return;
  }
  for (int64_t c0 = gwarp * 32; c0 < a.num_col; c0 += nwarps * 32) {
    const int64_t mine = c0 + lane;
    bool on = false;
    if (mine < a.num_col) {
      if (VK == VEC_EV_BOOL) on = static_cast<const uint8_t*>(a.vec)[mine] != 0;
      else on = __ldg(static_cast<const float*>(a.vec) + mine) != 0.0f;
    }
    unsigned act = __ballot_sync(0xffffffffu, on);
    while (act) {
      const int b = __ffs(act) - 1;
      act &= act - 1u;
      push_column(c0 + b, 1.0f);
    }
  }
}

// ---------------------------------------------------------------------------
// Taichi CPU algorithm: thread per owner
// ---------------------------------------------------------------------------
template <int KIND, int VK>
__global__ void __launch_bounds__(256) jc_pull_cpu_kernel(JcArgs a) {
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  const int32_t lim = (int32_t)a.num_col;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < a.num_row; row += nthr) {
    Lfsr88 key = lfsr88_key(a.seed + (uint32_t)row);
    int32_t c = (int32_t)lfsr88_start(key, a.fm);
    float r = 0.0f;
    while (c < lim) {
      const float w = jc_draw<KIND>(key, a.p0, a.p1);
      if (VK == VEC_EV_BOOL) {
        if (static_cast<const uint8_t*>(a.vec)[c]) r = __fadd_rn(r, w);
      } else if (VK == VEC_EV_F32) {
        if (__ldg(static_cast<const float*>(a.vec) + c) != 0.0f) r = __fadd_rn(r, w);
      } else {
        const float v = __ldg(static_cast<const float*>(a.vec) + c);
        if (KIND == JC_HOMO) r = __fadd_rn(r, v);
        else r = __fadd_rn(r, __fmul_rn(v, w));
      }
      c += (int32_t)lfsr88_inc(key, a.fm);
    }
    if (VK == VEC_DENSE && KIND == JC_HOMO) r = __fmul_rn(r, a.p0);
    a.out[row] = r;
  }
}

template <int KIND, int VK>
__global__ void __launch_bounds__(256) jc_push_cpu_kernel(JcArgs a) {
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  const int32_t lim = (int32_t)a.num_row;
  for (int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; col < a.num_col; col += nthr) {
    float cv = 1.0f;
    if (VK == VEC_EV_BOOL) {
      if (!static_cast<const uint8_t*>(a.vec)[col]) continue;
    } else if (VK == VEC_EV_F32) {
      if (__ldg(static_cast<const float*>(a.vec) + col) == 0.0f) continue;
    } else {
      cv = __ldg(static_cast<const float*>(a.vec) + col);
    }
    Lfsr88 key = lfsr88_key(a.seed + (uint32_t)col);
    int32_t r = (int32_t)lfsr88_start(key, a.fm);
    while (r < lim) {
      const float w = jc_draw<KIND>(key, a.p0, a.p1);
      float add;
      if (VK == VEC_DENSE) add = (KIND == JC_HOMO) ? __fmul_rn(cv, a.p0) : __fmul_rn(cv, w);
      else add = w;
      atomicAdd(a.out + r, add);
      r += (int32_t)lfsr88_inc(key, a.fm);
    }
  }
}

// ---------------------------------------------------------------------------
// materialisation of M (dense, row-major num_row x num_col) -- every connection written once
// ---------------------------------------------------------------------------
template <int KIND>
__global__ void __launch_bounds__(256) jc_dense_gpu_kernel(JcArgs a, int odp, float* dense) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t n_owner = odp ? a.num_row : a.num_col;
  const uint32_t lim = (uint32_t)(odp ? a.num_col : a.num_row);
  for (int64_t o = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); o < n_owner; o += nwarps) {
    const uint32_t i = (uint32_t)(o * 32 + lane);
    uint32_t c = a.step * (uint32_t)lane - 1u;
    uint32_t end = c + a.step;
    if (lim < end) end = lim;
    Lfsr88 key = lfsr88_key(a.seed + i);
    c += lfsr88_inc(key, a.fm);
    while (c < end) {
      const float w = jc_draw<KIND>(key, a.p0, a.p1);
      if (odp) dense[o * a.num_col + c] = w;
      else dense[(int64_t)c * a.num_col + o] = w;
      c += lfsr88_inc(key, a.fm);
    }
  }
}

template <int KIND>
__global__ void __launch_bounds__(256) jc_dense_cpu_kernel(JcArgs a, int odp, float* dense) {
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_owner = odp ? a.num_row : a.num_col;
  const int32_t lim = (int32_t)(odp ? a.num_col : a.num_row);
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_owner; o += nthr) {
    Lfsr88 key = lfsr88_key(a.seed + (uint32_t)o);
    int32_t c = (int32_t)lfsr88_start(key, a.fm);
    while (c < lim) {
      const float w = jc_draw<KIND>(key, a.p0, a.p1);
      if (odp) dense[o * a.num_col + c] = w;
      else dense[(int64_t)c * a.num_col + o] = w;
      c += (int32_t)lfsr88_inc(key, a.fm);
    }
  }
}

static int grid_warps(int64_t owners, int max_blocks) {
  int64_t g = (owners + 7) / 8;  // 8 warps per 256-thread block
  if (g < 1) g = 1;
  return (int)(g > max_blocks ? max_blocks : g);
}

static int grid_threads(int64_t owners, int max_blocks) {
  int64_t g = (owners + 255) / 256;
  if (g < 1) g = 1;
  return (int)(g > max_blocks ? max_blocks : g);
}

constexpr size_t kLaneBitsMax = 200 * 1024;  // shared-memory event bits of one lane's range

// the lane-major pull when the lane's column range fits shared memory
static bp_status launch_pull_homo_bool_lanes(const JcArgs& a, cudaStream_t st, bool& done) {
  done = false;
  const size_t bytes = (((size_t)a.step + 31) / 32) * sizeof(uint32_t);
  if (bytes > kLaneBitsMax) return BP_OK;
  static bool configured[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!configured[dev]) {
    BP_CUDA_TRY(cudaFuncSetAttribute(jc_pull_homo_bool_lanes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kLaneBitsMax));
    configured[dev] = true;
  }
  // blocks per lane: enough CTAs to fill the GPU; each loads its lane's bits once
  int64_t per_lane = ((int64_t)device_sm_count() * 8 + 31) / 32;
  int64_t rows_per_block = (a.num_row + per_lane - 1) / per_lane;
  if (rows_per_block < 256) rows_per_block = 256;
  per_lane = (a.num_row + rows_per_block - 1) / rows_per_block;
  BP_CUDA_TRY(cudaMemsetAsync(a.out, 0, sizeof(float) * (size_t)a.num_row, st));
  jc_pull_homo_bool_lanes_kernel<<<dim3((unsigned)per_lane, 32), 256, bytes, st>>>(a, rows_per_block);
  bp_status s = check_launch("jc_pull_homo_bool_lanes_kernel");
  if (s != BP_OK) return s;
  int64_t g = (a.num_row + 255) / 256;
  const int64_t maxb = (int64_t)device_sm_count() * 16;
  jc_counts_to_out_kernel<<<(unsigned)(g > maxb ? maxb : g), 256, 0, st>>>(a.out, a.num_row, a.p0);
  done = true;
  return check_launch("jc_counts_to_out_kernel");
}

template <int KIND, int VK>
static bp_status launch_mv(const JcArgs& a, int odp, int variant, cudaStream_t st) {
  const int maxb = device_sm_count() * 32;
  if (KIND == JC_HOMO && VK == VEC_EV_BOOL && odp && variant == BP_JC_TAICHI_GPU) {
    bool done = false;
    bp_status s = launch_pull_homo_bool_lanes(a, st, done);
    if (s != BP_OK || done) return s;
  }
  if (variant == BP_JC_TAICHI_GPU) {
    if (odp) jc_pull_gpu_kernel<KIND, VK><<<grid_warps(a.num_row, maxb), 256, 0, st>>>(a);
    else jc_push_gpu_kernel<KIND, VK><<<grid_warps(a.num_col, maxb), 256, 0, st>>>(a);
  } else {
    if (odp) jc_pull_cpu_kernel<KIND, VK><<<grid_threads(a.num_row, maxb), 256, 0, st>>>(a);
    else jc_push_cpu_kernel<KIND, VK><<<grid_threads(a.num_col, maxb), 256, 0, st>>>(a);
  }
  return check_launch("jitconn kernel");
}

template <int KIND>
static bp_status launch_mv_vk(const JcArgs& a, int vk, int odp, int variant, cudaStream_t st) {
  switch (vk) {
    case VEC_EV_BOOL: return launch_mv<KIND, VEC_EV_BOOL>(a, odp, variant, st);
    case VEC_EV_F32: return launch_mv<KIND, VEC_EV_F32>(a, odp, variant, st);
    default: return launch_mv<KIND, VEC_DENSE>(a, odp, variant, st);
  }
}

// ---------------------------------------------------------------------------
// The pull connectivity of one homogeneous projection, stored (Taichi GPU algorithm,
// outdim_parallel=1): for every input column c, the output rows whose lane streams visit c --
// the presynaptic-row CSR that the event-driven kernels stream, so that a network whose
// connectivity would be regenerated every step can be run from memory instead.  Stream
// (row, l) only visits stripe l, columns c with l * step <= c < min(l * step - 1 + step,
// num_col), so block (l, part) owns one part [lo, hi) of that stripe (at most kJcCsrWidth
// columns, a 32-bit counter each in shared memory) and walks the lane-l stream of every row
// up to hi.  PASS 0 counts each owned column's rows into counts[c]; PASS 1 writes
// row + row_offset at base[c] + the row's rank among the column's rows (a shared-memory
// cursor: the order inside a column is the order the threads reach it); a position at or past
// nnz (a base inconsistent with the counts) is skipped.
// ---------------------------------------------------------------------------
constexpr uint32_t kJcCsrWidth = 49152;  // 192 KB of counters

template <int PASS, typename IdxT>
__global__ void __launch_bounds__(1024, 1) jc_csr_kernel(JcArgs a, uint32_t parts, uint32_t width,
                                                          uint32_t* __restrict__ counts,
                                                          const int64_t* __restrict__ base, int64_t row_offset,
                                                          IdxT* __restrict__ indices, int64_t nnz) {
  extern __shared__ uint32_t cnt[];
  const uint32_t l = blockIdx.x / parts, part = blockIdx.x % parts;
  const uint32_t lim = (uint32_t)a.num_col;
  uint32_t end = a.step * l - 1u + a.step;  // the streams' bound (uint32, as in the pull kernels)
  if (lim < end) end = lim;
  const uint32_t lo = a.step * l + part * width;
  if (lo >= end) return;
  const uint32_t hi = end - lo < width ? end : lo + width;
  for (uint32_t j = threadIdx.x; j < hi - lo; j += blockDim.x) cnt[j] = 0u;
  __syncthreads();
  for (int64_t row = threadIdx.x; row < a.num_row; row += blockDim.x) {
    Lfsr88 key = lfsr88_key(a.seed + (uint32_t)(row * 32 + l));
    uint32_t c = a.step * l - 1u;
    c += lfsr88_inc(key, a.fm);
    while (c < hi) {
      if (c >= lo) {
        const uint32_t r = atomicAdd(&cnt[c - lo], 1u);
        if (PASS == 1) {
          const int64_t at = base[c] + (int64_t)r;
          if (at >= 0 && at < nnz) indices[at] = (IdxT)(row + row_offset);
        }
      }
      c += lfsr88_inc(key, a.fm);
    }
  }
  if (PASS == 0) {
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < hi - lo; j += blockDim.x) counts[lo + j] = cnt[j];
  }
}

static bp_status jc_common_checks(int32_t kind, int64_t num_row, int64_t num_col, int32_t clen, int32_t variant,
                                  const char* who) {
  BP_REQUIRE(kind >= BP_JC_HOMO && kind <= BP_JC_NORMAL, BP_EINVAL, "%s: bad kind %d", who, (int)kind);
  BP_REQUIRE(variant == BP_JC_TAICHI_GPU || variant == BP_JC_TAICHI_CPU, BP_EINVAL, "%s: bad variant %d", who,
             (int)variant);
  BP_REQUIRE(num_row >= 0 && num_col >= 0, BP_EINVAL, "%s: negative size", who);
  // the reference's kernels index with int32 loop counters over owner*32 + lane
  BP_REQUIRE(num_row * 32 < INT32_MAX && num_col * 32 < INT32_MAX, BP_ENOTSUP,
             "%s: dimensions beyond the reference's int32 stream indexing", who);
  BP_REQUIRE(clen >= 1, BP_EINVAL, "%s: conn_len must be >= 1 (got %d)", who, (int)clen);
  return BP_OK;
}

static JcArgs make_args(const void* vec, float* out, int64_t num_row, int64_t num_col, float p0, float p1,
                        int32_t clen, uint32_t seed) {
  JcArgs a;
  a.vec = vec;
  a.out = out;
  a.num_row = num_row;
  a.num_col = num_col;
  a.p0 = p0;
  a.p1 = p1;
  a.fm = make_fastmod((uint32_t)clen);
  a.seed = seed;
  const int32_t sh = ((int32_t)num_row + 1) >> 5;
  a.step = (uint32_t)(sh > 1 ? sh : 1);
  return a;
}

}  // namespace bp

using namespace bp;

extern "C" {

bp_status bp_jitconn_mv(bp_jc_kind kind, bp_jc_vec vec_kind, const void* vec, int64_t num_col, int64_t num_row,
                        float p0, float p1, int32_t clen, uint32_t seed, int32_t outdim_parallel,
                        bp_jc_variant variant, float* out, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  bp_status s = jc_common_checks(kind, num_row, num_col, clen, variant, "jitconn_mv");
  if (s != BP_OK) return s;
  BP_REQUIRE(vec_kind >= BP_VEC_EVENT_BOOL && vec_kind <= BP_VEC_DENSE_F32, BP_EDTYPE, "jitconn_mv: bad vec kind %d",
             (int)vec_kind);
  if (num_row == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "jitconn_mv: null out");
  const bool push = !outdim_parallel;
  if (push || num_col == 0) BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)num_row, st));
  if (num_col == 0) return BP_OK;
  BP_REQUIRE(vec != nullptr, BP_EINVAL, "jitconn_mv: null vector");
  JcArgs a = make_args(vec, out, num_row, num_col, p0, p1, clen, seed);
  ScopedKernelTimer tk(st);
  switch (kind) {
    case BP_JC_HOMO: return launch_mv_vk<JC_HOMO>(a, vec_kind, outdim_parallel ? 1 : 0, variant, st);
    case BP_JC_UNIFORM: return launch_mv_vk<JC_UNIFORM>(a, vec_kind, outdim_parallel ? 1 : 0, variant, st);
    default: return launch_mv_vk<JC_NORMAL>(a, vec_kind, outdim_parallel ? 1 : 0, variant, st);
  }
}

bp_status bp_jitconn_dense(bp_jc_kind kind, float p0, float p1, int32_t clen, uint32_t seed, int64_t num_row,
                           int64_t num_col, int32_t outdim_parallel, bp_jc_variant variant, float* dense,
                           bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  bp_status s = jc_common_checks(kind, num_row, num_col, clen, variant, "jitconn_dense");
  if (s != BP_OK) return s;
  if (num_row == 0 || num_col == 0) return BP_OK;
  BP_REQUIRE(dense != nullptr, BP_EINVAL, "jitconn_dense: null output");
  BP_CUDA_TRY(cudaMemsetAsync(dense, 0, sizeof(float) * (size_t)num_row * (size_t)num_col, st));
  JcArgs a = make_args(nullptr, nullptr, num_row, num_col, p0, p1, clen, seed);
  const int odp = outdim_parallel ? 1 : 0;
  const int64_t owners = odp ? num_row : num_col;
  const int maxb = device_sm_count() * 32;
  if (variant == BP_JC_TAICHI_GPU) {
    const int g = grid_warps(owners, maxb);
    if (kind == BP_JC_HOMO) jc_dense_gpu_kernel<JC_HOMO><<<g, 256, 0, st>>>(a, odp, dense);
    else if (kind == BP_JC_UNIFORM) jc_dense_gpu_kernel<JC_UNIFORM><<<g, 256, 0, st>>>(a, odp, dense);
    else jc_dense_gpu_kernel<JC_NORMAL><<<g, 256, 0, st>>>(a, odp, dense);
  } else {
    const int g = grid_threads(owners, maxb);
    if (kind == BP_JC_HOMO) jc_dense_cpu_kernel<JC_HOMO><<<g, 256, 0, st>>>(a, odp, dense);
    else if (kind == BP_JC_UNIFORM) jc_dense_cpu_kernel<JC_UNIFORM><<<g, 256, 0, st>>>(a, odp, dense);
    else jc_dense_cpu_kernel<JC_NORMAL><<<g, 256, 0, st>>>(a, odp, dense);
  }
  return check_launch("jitconn_dense kernel");
}

bp_status bp_jitconn_csr(int32_t pass, int32_t clen, uint32_t seed, int64_t num_row, int64_t num_col,
                         uint32_t* counts, const int64_t* base, int64_t row_offset, void* indices, int64_t nnz,
                         bp_itype itype, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  bp_status s = jc_common_checks(BP_JC_HOMO, num_row, num_col, clen, BP_JC_TAICHI_GPU, "jitconn_csr");
  if (s != BP_OK) return s;
  BP_REQUIRE(pass == 0 || pass == 1, BP_EINVAL, "jitconn_csr: pass must be 0 or 1 (got %d)", (int)pass);
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "jitconn_csr: bad index type %d", (int)itype);
  BP_REQUIRE(row_offset >= 0 && (itype == BP_I64 || row_offset + num_row <= (int64_t)INT32_MAX), BP_EINVAL,
             "jitconn_csr: row ids up to %lld do not fit the index type", (long long)(row_offset + num_row));
  if (num_row == 0 || num_col == 0) {
    if (pass == 0 && num_col > 0) {
      BP_REQUIRE(counts != nullptr, BP_EINVAL, "jitconn_csr: null counts");
      BP_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(uint32_t) * (size_t)num_col, st));
    }
    return BP_OK;
  }
  BP_REQUIRE(pass == 1 || counts != nullptr, BP_EINVAL, "jitconn_csr: pass 0 needs counts");
  BP_REQUIRE(pass == 0 || (base != nullptr && indices != nullptr && nnz >= 0), BP_EINVAL,
             "jitconn_csr: pass 1 needs base and indices");
  JcArgs a = make_args(nullptr, nullptr, num_row, num_col, 1.0f, 0.0f, clen, seed);
  // columns the streams never reach (beyond 32 stripes) keep a count of 0
  if (pass == 0) BP_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(uint32_t) * (size_t)num_col, st));
  const uint32_t parts = (a.step + kJcCsrWidth - 1) / kJcCsrWidth;
  const uint32_t width = (a.step + parts - 1) / parts;
  const size_t smem = sizeof(uint32_t) * (size_t)width;
  const dim3 grid(32 * parts);
  static bool configured[64][4] = {};
  int dev = 0;
  BP_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) dev = 0;
  const int which = pass * 2 + (itype == BP_I64 ? 1 : 0);
  if (!configured[dev][which]) {
    const int lim = (int)(sizeof(uint32_t) * kJcCsrWidth);
    cudaError_t e;
    if (which == 0) e = cudaFuncSetAttribute(jc_csr_kernel<0, int32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    else if (which == 1) e = cudaFuncSetAttribute(jc_csr_kernel<0, int64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    else if (which == 2) e = cudaFuncSetAttribute(jc_csr_kernel<1, int32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    else e = cudaFuncSetAttribute(jc_csr_kernel<1, int64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    BP_CUDA_TRY(e);
    configured[dev][which] = true;
  }
  if (pass == 0) {
    if (itype == BP_I64) jc_csr_kernel<0, int64_t><<<grid, 1024, smem, st>>>(a, parts, width, counts, nullptr, 0, nullptr, 0);
    else jc_csr_kernel<0, int32_t><<<grid, 1024, smem, st>>>(a, parts, width, counts, nullptr, 0, nullptr, 0);
  } else if (itype == BP_I64) {
    jc_csr_kernel<1, int64_t><<<grid, 1024, smem, st>>>(a, parts, width, nullptr, base, row_offset,
                                                         static_cast<int64_t*>(indices), nnz);
  } else {
    jc_csr_kernel<1, int32_t><<<grid, 1024, smem, st>>>(a, parts, width, nullptr, base, row_offset,
                                                         static_cast<int32_t*>(indices), nnz);
  }
  return check_launch("jc_csr_kernel");
}

}  // extern "C"
