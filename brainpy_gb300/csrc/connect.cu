// connect.cu -- FixedProb connectivity built on the device.
//
// Reference: brainpy/_src/connect/random_conn.py:73-128 (FixedProb._iii / build_csr).  Every
// selected pre-synaptic row gets K = int(post_num * prob) post-synaptic columns: K distinct
// columns drawn uniformly without replacement (numba's rng.choice(post_num, K, replace=False)),
// or, with allow_multi_conn, K independent uniform draws; with include_self=False the diagonal
// entries that were drawn are then removed, so such a row is one shorter.
//
// The reference's numba RNG cannot be reproduced; the distribution is.  Row r's columns are the
// first K distinct values of the sequence u_r(0), u_r(1), ... of independent uniform draws on
// [0, n) (a counter-based hash of (seed, r, t), mapped with a 64-bit multiply-high): the first K
// distinct values of an i.i.d. uniform sequence are a uniformly random K-subset, in a uniformly
// random order -- the same law as the prefix of a random permutation.
//
// One warp per row.  Draws go 32 at a time (lane l takes t0 + l); a lane's value is new when no
// lower lane of the batch drew it (__match_any_sync) and the row's hash set (shared memory,
// 2K..4K slots per warp) does not hold it; the new values are ranked by lane, and as many as the
// row still needs are kept -- exactly the sequential "first K distinct" rule.
#include "common.cuh"
#include "timer.cuh"

namespace bp {

constexpr int kConnMaxWarps = 4;                 // warps (rows in flight) per CTA, at most
constexpr int kConnMaxK = 16384;                 // distinct draws per row held in shared memory
constexpr size_t kConnSmemBudget = 200 * 1024;   // hash sets of one CTA

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // SplitMix64 finaliser (Steele et al. 2014)
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return x;
}

// u_r(t): uniform on [0, n)
__device__ __forceinline__ uint32_t conn_draw(uint64_t seed_key, uint64_t row, uint64_t t, uint32_t n) {
  const uint64_t h = mix64(seed_key + row * 0xD1B54A32D192ED03ull + t * 0x8CB92BA72F3D8DD7ull);
  return (uint32_t)__umul64hi(h, (uint64_t)n);
}

__host__ __device__ __forceinline__ uint64_t conn_seed_key(uint64_t seed) {
  return (seed + 1ull) * 0x9E3779B97F4A7C15ull;
}

__device__ __forceinline__ uint32_t slot_of(uint32_t v, uint32_t hmask) { return (v * 2654435761u) & hmask; }

// true when v+1 is stored (linear probing; 0 = empty)
__device__ __forceinline__ bool set_has(const uint32_t* tab, uint32_t hmask, uint32_t v) {
  uint32_t s = slot_of(v, hmask);
  for (;;) {
    const uint32_t x = tab[s];
    if (x == 0u) return false;
    if (x == v + 1u) return true;
    s = (s + 1u) & hmask;
  }
}

__device__ __forceinline__ void set_put(uint32_t* tab, uint32_t hmask, uint32_t v) {
  uint32_t s = slot_of(v, hmask);
  for (;;) {
    const uint32_t old = atomicCAS(tab + s, 0u, v + 1u);
    if (old == 0u || old == v + 1u) return;
    s = (s + 1u) & hmask;
  }
}

// Generates row `row`: calls emit(pos, value) for the kept values in order (pos = 0..K-1) and
// returns the row's length after the self-connection removal, or -1 when the draw count passes
// a bound far above what K distinct values out of n need (n (ln n + 1) on average at K = n), so
// that a defect can never keep the warp looping.  All lanes of the warp call it.
template <bool MULTI, typename Emit>
__device__ __forceinline__ int conn_row(uint64_t seed_key, int64_t row, uint32_t n, int K, bool drop_self,
                                        uint32_t* tab, uint32_t hmask, Emit emit) {
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  const uint64_t max_draws = 64ull * (uint64_t)K + 32ull * (uint64_t)n + 65536ull;
  int count = 0, kept = 0;
  for (uint64_t t0 = 0; count < K; t0 += 32) {
    if (t0 > max_draws) return -1;
    const uint32_t v = conn_draw(seed_key, (uint64_t)row, t0 + (uint64_t)lane, n);
    bool cand = true;
    if (!MULTI) {
      const uint32_t same = __match_any_sync(0xffffffffu, v);
      cand = ((same & lt) == 0u) && !set_has(tab, hmask, v);
    }
    const uint32_t cb = __ballot_sync(0xffffffffu, cand);
    const bool take = cand && __popc(cb & lt) < K - count;  // the first K - count new values
    const bool self = take && drop_self && (int64_t)v == row;
    const uint32_t tb = __ballot_sync(0xffffffffu, take);
    const uint32_t sb = __ballot_sync(0xffffffffu, self);
    if (take) {
      if (!MULTI) set_put(tab, hmask, v);
      // position among the kept values (self connections removed)
      if (!self) emit(kept + __popc(tb & lt) - __popc(sb & lt), v);
    }
    count += __popc(tb);
    kept += __popc(tb) - __popc(sb);
    __syncwarp();
  }
  return kept;
}

// Empties the warp's hash set.
__device__ __forceinline__ void set_clear_all(uint32_t* tab, uint32_t hsize) {
  const int lane = threadIdx.x & 31;
  for (uint32_t s = lane; s < hsize; s += 32) tab[s] = 0u;
  __syncwarp();
}

template <bool MULTI, bool FILL>
__global__ void __launch_bounds__(32 * kConnMaxWarps) fixed_prob_kernel(int64_t m, uint32_t n, int K, uint64_t seed_key,
                                                                      int drop_self, const uint8_t* __restrict__ row_mask,
                                                                      const int64_t* __restrict__ indptr,
                                                                      int32_t* __restrict__ out, uint32_t hsize) {
  extern __shared__ uint32_t conn_tab[];
  const int warp = threadIdx.x >> 5;
  uint32_t* tab = conn_tab + (size_t)warp * hsize;
  const uint32_t hmask = hsize - 1u;
  if (!MULTI) set_clear_all(tab, hsize);
  const int wpc = blockDim.x >> 5;
  const int64_t nwarps = (int64_t)gridDim.x * wpc;
  for (int64_t row = (int64_t)blockIdx.x * wpc + warp; row < m; row += nwarps) {
    if (row_mask && !row_mask[row]) {
      if (!FILL && (threadIdx.x & 31) == 0) out[row] = 0;
      continue;
    }
    if (FILL) {
      int32_t* dst = out + indptr[row];
      const int len = conn_row<MULTI>(seed_key, row, n, K, drop_self != 0, tab, hmask,
                                      [&](int pos, uint32_t v) { dst[pos] = (int32_t)v; });
      if (len < 0 && (threadIdx.x & 31) == 0) dst[0] = -1;  // the caller checks indices >= 0
    } else {
      const int len = conn_row<MULTI>(seed_key, row, n, K, drop_self != 0, tab, hmask, [](int, uint32_t) {});
      if ((threadIdx.x & 31) == 0) out[row] = len;
    }
    if (!MULTI) set_clear_all(tab, hsize);
  }
}

static uint32_t hash_slots(int K) {
  uint32_t h = 64;
  while (h < 2u * (uint32_t)K) h <<= 1;
  return h;
}

template <bool FILL>
static bp_status launch_fixed_prob(int64_t m, int64_t n, int32_t K, uint64_t seed, int allow_multi, int drop_self,
                                   const uint8_t* row_mask, const int64_t* indptr, int32_t* out, cudaStream_t st) {
  const uint32_t hsize = allow_multi ? 0u : hash_slots(K);
  int wpc = kConnMaxWarps;  // rows per CTA: as many hash sets as the shared-memory budget holds
  while (wpc > 1 && (size_t)hsize * wpc * sizeof(uint32_t) > kConnSmemBudget) --wpc;
  const size_t smem = (size_t)hsize * wpc * sizeof(uint32_t);
  int64_t blocks = (m + wpc - 1) / wpc;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  const uint64_t key = conn_seed_key(seed);
  if (allow_multi) {
    fixed_prob_kernel<true, FILL><<<(unsigned)blocks, 32 * wpc, 0, st>>>(m, (uint32_t)n, K, key, drop_self, row_mask,
                                                                         indptr, out, 0);
  } else {
    auto kfn = fixed_prob_kernel<false, FILL>;
    BP_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kConnSmemBudget));
    kfn<<<(unsigned)blocks, 32 * wpc, smem, st>>>(m, (uint32_t)n, K, key, drop_self, row_mask, indptr, out, hsize);
  }
  return check_launch("fixed_prob_kernel");
}

static bp_status fixed_prob_check(const char* who, int64_t m, int64_t n, int32_t K, int allow_multi, int include_self) {
  BP_REQUIRE(m >= 0 && n >= 0, BP_EINVAL, "%s: negative size", who);
  BP_REQUIRE(n <= (int64_t)UINT32_MAX / 2 && m <= INT32_MAX, BP_ENOTSUP, "%s: sizes beyond int32 range", who);
  BP_REQUIRE(K >= 0 && (allow_multi || K <= n), BP_EINVAL, "%s: %d distinct columns out of %lld", who, K,
             (long long)n);
  BP_REQUIRE(allow_multi || K <= kConnMaxK, BP_ENOTSUP,
             "%s: %d distinct columns per row; at most %d are supported without allow_multi_conn", who, K, kConnMaxK);
  BP_REQUIRE(include_self || m == n, BP_EINVAL, "%s: include_self=False needs pre_num == post_num (%lld != %lld)", who,
             (long long)m, (long long)n);
  return BP_OK;
}

// true when p is memory the device can write (device or managed): the generator is a setup
// call, so it checks its output pointers instead of faulting on host addresses
static bool device_writable(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace bp

using namespace bp;

extern "C" {

bp_status bp_fixed_prob_row_lengths(int64_t m, int64_t n, int32_t K, uint64_t seed, int32_t allow_multi,
                                    int32_t include_self, const uint8_t* row_mask, int32_t* lengths,
                                    bp_stream_t stream) {
  clear_error();
  bp_status s = fixed_prob_check("fixed_prob_row_lengths", m, n, K, allow_multi, include_self);
  if (s != BP_OK || m == 0) return s;
  BP_REQUIRE(lengths != nullptr, BP_EINVAL, "fixed_prob_row_lengths: null lengths");
  BP_REQUIRE(device_writable(lengths) && (!row_mask || device_writable(row_mask)), BP_EINVAL,
             "fixed_prob_row_lengths: lengths and row_mask must be device memory");
  cudaStream_t st = as_cuda(stream);
  if (K == 0 || n == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(lengths, 0, sizeof(int32_t) * (size_t)m, st));
    return BP_OK;
  }
  return launch_fixed_prob<false>(m, n, K, seed, allow_multi, include_self ? 0 : 1, row_mask, nullptr, lengths, st);
}

bp_status bp_fixed_prob_fill(int64_t m, int64_t n, int32_t K, uint64_t seed, int32_t allow_multi,
                             int32_t include_self, const uint8_t* row_mask, const int64_t* indptr, int32_t* indices,
                             bp_stream_t stream) {
  clear_error();
  bp_status s = fixed_prob_check("fixed_prob_fill", m, n, K, allow_multi, include_self);
  if (s != BP_OK || m == 0 || K == 0 || n == 0) return s;
  BP_REQUIRE(indptr && indices, BP_EINVAL, "fixed_prob_fill: null indptr/indices");
  BP_REQUIRE(device_writable(indices) && device_writable(indptr) && (!row_mask || device_writable(row_mask)),
             BP_EINVAL, "fixed_prob_fill: indptr, indices and row_mask must be device memory");
  ScopedKernelTimer tk(as_cuda(stream));
  return launch_fixed_prob<true>(m, n, K, seed, allow_multi, include_self ? 0 : 1, row_mask, indptr, indices,
                                 as_cuda(stream));
}

}  // extern "C"
