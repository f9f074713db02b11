// csrmv.cu -- sparse.csrmv on plain CSR (dense float32 vector).
//
// transpose=0: y[i] = sum_j A[i, j] x[j]   one warp per row, coalesced index/weight streaming,
//              gathers of x, lane partials reduced in the warp (deterministic order).
// transpose=1: y[j] = sum_i A[i, j] x[i]   one warp per row with x[i] != 0, red.global.add.f32.
//              (bp_csrmv_planned is the shared-memory tiled form of the same product.)
// Homogeneous weight: x values are summed and multiplied by w once per lane, as the reference's
// Taichi GPU kernels do (brainpy/_src/math/sparse/_csr_mv_taichi.py:115-120, :124-135).
// Reference semantics: brainpy/_src/math/sparse/_csr_mv.py:126-164 (Numba CPU).
#include "common.cuh"
#include "timer.cuh"

namespace bp {

template <typename IdxT>
__device__ __forceinline__ void csr_row_bounds(const IdxT* indptr, int64_t row, int64_t nnz, int64_t& b, int64_t& e) {
  b = (int64_t)indptr[row];
  e = (int64_t)indptr[row + 1];
  b = b < 0 ? 0 : (b > nnz ? nnz : b);
  e = e < b ? b : (e > nnz ? nnz : e);
}

constexpr int kNUnroll = 8;

template <typename IdxT, bool HOMO>
__global__ void __launch_bounds__(256) csrmv_n_kernel(const IdxT* __restrict__ indptr, const IdxT* __restrict__ indices,
                                                      const float* __restrict__ data, int64_t nnz, int64_t m,
                                                      int64_t n, const float* __restrict__ x, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < m; row += nwarps) {
    int64_t b, e;
    csr_row_bounds(indptr, row, nnz, b, e);
    float acc = 0.0f;
    int64_t j = b + lane;
    // kNUnroll entries per lane in flight (index loads, then the gathers), summed in j order
    for (; j + 32 * (kNUnroll - 1) < e; j += 32 * kNUnroll) {
      int64_t c[kNUnroll];
      float xv[kNUnroll];
#pragma unroll
      for (int u = 0; u < kNUnroll; ++u) c[u] = (int64_t)indices[j + 32 * u];
#pragma unroll
      for (int u = 0; u < kNUnroll; ++u) xv[u] = (uint64_t)c[u] < (uint64_t)n ? __ldg(x + c[u]) : 0.0f;
#pragma unroll
      for (int u = 0; u < kNUnroll; ++u) {
        if (HOMO) acc += xv[u];
        else acc = fmaf(data[j + 32 * u], xv[u], acc);
      }
    }
    // the rest of the row (< 32 * kNUnroll entries): up to 4 entries per lane in flight a
    // round, predicated, still summed in j order
    for (; j < e; j += 32 * 4) {
      int64_t c[4];
      float xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) c[u] = j + 32 * u < e ? (int64_t)indices[j + 32 * u] : -1;
#pragma unroll
      for (int u = 0; u < 4; ++u) xv[u] = (uint64_t)c[u] < (uint64_t)n ? __ldg(x + c[u]) : 0.0f;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (j + 32 * u < e) {
          if (HOMO) acc += xv[u];
          else acc = fmaf(data[j + 32 * u], xv[u], acc);
        }
      }
    }
    if (HOMO) acc *= __ldg(data);
    acc = warp_sum(acc);
    if (lane == 0) out[row] = acc;
  }
}

template <typename IdxT, bool HOMO>
__global__ void __launch_bounds__(256) csrmv_t_kernel(const IdxT* __restrict__ indptr, const IdxT* __restrict__ indices,
                                                      const float* __restrict__ data, int64_t nnz, int64_t m,
                                                      int64_t n, const float* __restrict__ x, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < m; row += nwarps) {
    const float xv = __ldg(x + row);
    if (xv == 0.0f) continue;  // warp-uniform: the row adds nothing
    int64_t b, e;
    csr_row_bounds(indptr, row, nnz, b, e);
    const float wx = HOMO ? __fmul_rn(__ldg(data), xv) : 0.0f;
    for (int64_t j = b + lane; j < e; j += 32) {
      int64_t c = (int64_t)indices[j];
      if ((uint64_t)c < (uint64_t)n) atomicAdd(out + c, HOMO ? wx : __fmul_rn(data[j], xv));
    }
  }
}

// CSR -> COO rows (brainpy/_src/math/sparse/_utils.py:44-52): rows[j] = i for j in row i
template <typename IdxT>
__global__ void __launch_bounds__(256) csr_rows_kernel(const IdxT* __restrict__ indptr, int64_t m, int64_t nnz,
                                                       IdxT* __restrict__ rows) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < m; row += nwarps) {
    int64_t b, e;
    csr_row_bounds(indptr, row, nnz, b, e);
    for (int64_t j = b + lane; j < e; j += 32) rows[j] = (IdxT)row;
  }
}

// CSR -> dense (brainpy/_src/math/sparse/_utils.py:70-81 and :101-114): duplicates add up
template <typename IdxT>
__global__ void __launch_bounds__(256) csr_dense_kernel(const float* __restrict__ data, int homo,
                                                        const IdxT* __restrict__ indptr, const IdxT* __restrict__ indices,
                                                        int64_t m, int64_t n, int64_t nnz, float* __restrict__ dense) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < m; row += nwarps) {
    int64_t b, e;
    csr_row_bounds(indptr, row, nnz, b, e);
    for (int64_t j = b + lane; j < e; j += 32) {
      const int64_t c = (int64_t)indices[j];
      if ((uint64_t)c < (uint64_t)n) atomicAdd(dense + row * n + c, homo ? __ldg(data) : data[j]);
    }
  }
}

// The weight cotangent of the CSR products (brainpy/_src/math/event/_csr_matvec.py:545-547,
// brainpy/_src/math/sparse/_csr_mv.py:237-239): out[j] = x[i] * y[indices[j]] for every stored
// entry j of row i, 0 where the column is out of range.  One warp per row, coalesced index
// stream and output, gathers of y.  Entries outside every row ([0, indptr[0]) and
// [indptr[m], nnz)) are set to 0.
template <typename IdxT>
__global__ void __launch_bounds__(256) csr_sampled_outer_kernel(const IdxT* __restrict__ indptr,
                                                                const IdxT* __restrict__ indices, int64_t nnz,
                                                                int64_t m, int64_t n, const float* __restrict__ x,
                                                                const float* __restrict__ y, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (gw == 0) {
    int64_t b0 = (int64_t)indptr[0], em = (int64_t)indptr[m];
    b0 = b0 < 0 ? 0 : (b0 > nnz ? nnz : b0);
    em = em < b0 ? b0 : (em > nnz ? nnz : em);
    for (int64_t j = lane; j < b0; j += 32) out[j] = 0.0f;
    for (int64_t j = em + lane; j < nnz; j += 32) out[j] = 0.0f;
  }
  for (int64_t row = gw; row < m; row += nwarps) {
    int64_t b, e;
    csr_row_bounds(indptr, row, nnz, b, e);
    const float xv = __ldg(x + row);
    for (int64_t j = b + lane; j < e; j += 32) {
      const int64_t c = (int64_t)indices[j];
      out[j] = (uint64_t)c < (uint64_t)n ? __fmul_rn(xv, __ldg(y + c)) : 0.0f;
    }
  }
}

static int grid_rows(int64_t m) {
  int64_t g = (m + 7) / 8;
  const int64_t maxb = (int64_t)device_sm_count() * 32;
  if (g < 1) g = 1;
  return (int)(g > maxb ? maxb : g);
}

template <typename IdxT>
static bp_status csrmv_dispatch(const float* data, bool homo, const IdxT* indices, const IdxT* indptr, int64_t nnz,
                                const float* x, int64_t m, int64_t n, int transpose, float* out, cudaStream_t st) {
  const int g = grid_rows(m);
  ScopedKernelTimer tk(st);
  if (transpose) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n, st));
    if (homo) csrmv_t_kernel<IdxT, true><<<g, 256, 0, st>>>(indptr, indices, data, nnz, m, n, x, out);
    else csrmv_t_kernel<IdxT, false><<<g, 256, 0, st>>>(indptr, indices, data, nnz, m, n, x, out);
  } else {
    if (homo) csrmv_n_kernel<IdxT, true><<<g, 256, 0, st>>>(indptr, indices, data, nnz, m, n, x, out);
    else csrmv_n_kernel<IdxT, false><<<g, 256, 0, st>>>(indptr, indices, data, nnz, m, n, x, out);
  }
  return check_launch("csrmv kernel");
}

}  // namespace bp

using namespace bp;

extern "C" {

bp_status bp_csrmv(const float* data, int64_t ndata, const void* indices, const void* indptr, bp_itype itype,
                   int64_t nnz, const float* vec, int64_t m, int64_t n, int32_t transpose, float* out,
                   bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(m >= 0 && n >= 0 && nnz >= 0, BP_EINVAL, "csrmv: negative size");
  BP_REQUIRE(m <= INT32_MAX && n <= INT32_MAX, BP_ENOTSUP, "csrmv: dimensions beyond int32 range");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "csrmv: bad index type %d", (int)itype);
  BP_REQUIRE(ndata == 1 || ndata == nnz, BP_ESHAPE,
             "csrmv: the size of data should be 1 or be consistent with indices (%lld vs %lld)", (long long)ndata,
             (long long)nnz);
  const int64_t n_out = transpose ? n : m;
  if (n_out == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "csrmv: null out");
  if (m == 0 || nnz == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n_out, st));
    return BP_OK;
  }
  BP_REQUIRE(data && indices && indptr && vec, BP_EINVAL, "csrmv: null data/indices/indptr/vector");
  const bool homo = ndata == 1;
  if (itype == BP_I32)
    return csrmv_dispatch<int32_t>(data, homo, static_cast<const int32_t*>(indices), static_cast<const int32_t*>(indptr),
                                   nnz, vec, m, n, transpose, out, st);
  return csrmv_dispatch<int64_t>(data, homo, static_cast<const int64_t*>(indices), static_cast<const int64_t*>(indptr),
                                 nnz, vec, m, n, transpose, out, st);
}

}  // extern "C"

extern "C" {

bp_status bp_csr_sampled_outer(const float* x, const float* y, const void* indices, const void* indptr,
                               bp_itype itype, int64_t nnz, int64_t m, int64_t n, float* out, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(m >= 0 && n >= 0 && nnz >= 0, BP_EINVAL, "csr_sampled_outer: negative size");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "csr_sampled_outer: bad index type %d", (int)itype);
  if (nnz == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "csr_sampled_outer: null out");
  if (m == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)nnz, st));
    return BP_OK;
  }
  BP_REQUIRE(x && indices && indptr && (y || n == 0), BP_EINVAL, "csr_sampled_outer: null pointer");
  const int g = grid_rows(m);
  ScopedKernelTimer tk(st);
  if (itype == BP_I32)
    csr_sampled_outer_kernel<int32_t><<<g, 256, 0, st>>>(static_cast<const int32_t*>(indptr),
                                                         static_cast<const int32_t*>(indices), nnz, m, n, x, y, out);
  else
    csr_sampled_outer_kernel<int64_t><<<g, 256, 0, st>>>(static_cast<const int64_t*>(indptr),
                                                         static_cast<const int64_t*>(indices), nnz, m, n, x, y, out);
  return check_launch("csr_sampled_outer_kernel");
}

bp_status bp_csr_to_coo(const void* indptr, bp_itype itype, int64_t m, int64_t nnz, void* rows, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(m >= 0 && nnz >= 0, BP_EINVAL, "csr_to_coo: negative size");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "csr_to_coo: bad index type");
  if (m == 0 || nnz == 0) return BP_OK;
  BP_REQUIRE(indptr && rows, BP_EINVAL, "csr_to_coo: null pointer");
  const int g = grid_rows(m);
  if (itype == BP_I32)
    csr_rows_kernel<int32_t><<<g, 256, 0, st>>>(static_cast<const int32_t*>(indptr), m, nnz, static_cast<int32_t*>(rows));
  else
    csr_rows_kernel<int64_t><<<g, 256, 0, st>>>(static_cast<const int64_t*>(indptr), m, nnz, static_cast<int64_t*>(rows));
  return check_launch("csr_rows_kernel");
}

bp_status bp_csr_to_dense(const float* data, int64_t ndata, const void* indices, const void* indptr, bp_itype itype,
                          int64_t nnz, int64_t m, int64_t n, float* dense, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(m >= 0 && n >= 0 && nnz >= 0, BP_EINVAL, "csr_to_dense: negative size");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "csr_to_dense: bad index type");
  BP_REQUIRE(ndata == 1 || ndata == nnz, BP_ESHAPE, "csr_to_dense: data size %lld vs nnz %lld", (long long)ndata,
             (long long)nnz);
  if (m == 0 || n == 0) return BP_OK;
  BP_REQUIRE(dense != nullptr, BP_EINVAL, "csr_to_dense: null output");
  BP_CUDA_TRY(cudaMemsetAsync(dense, 0, sizeof(float) * (size_t)m * (size_t)n, st));
  if (nnz == 0) return BP_OK;
  BP_REQUIRE(data && indices && indptr, BP_EINVAL, "csr_to_dense: null pointer");
  const int g = grid_rows(m);
  if (itype == BP_I32)
    csr_dense_kernel<int32_t><<<g, 256, 0, st>>>(data, ndata == 1, static_cast<const int32_t*>(indptr),
                                                 static_cast<const int32_t*>(indices), m, n, nnz, dense);
  else
    csr_dense_kernel<int64_t><<<g, 256, 0, st>>>(data, ndata == 1, static_cast<const int64_t*>(indptr),
                                                 static_cast<const int64_t*>(indices), m, n, nnz, dense);
  return check_launch("csr_dense_kernel");
}

}  // extern "C"
