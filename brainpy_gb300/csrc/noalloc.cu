// noalloc.cu -- event.csrmv without any allocation by the caller or the library.
//
// Who needs it: a caller that can hand the operator nothing but its operands and its
// result buffer.  The reference's own binding is such a caller: a legacy XLA custom
// call receives its operand and result buffers from XLA and has no scratch allocator to
// ask for more, and calling cudaMalloc from inside it would synchronise the device in
// the middle of XLA's asynchronous stream.  The same holds for code that runs with a
// fixed memory budget after start-up and may not allocate on its step path.
//
// How: the event-driven (transpose) path needs scratch for the list of active rows and
// their count.  Here that scratch is one file-scope __device__ array, so it exists in
// every GPU's copy of this module for as long as the library stays loaded, and this
// entry point calls no cudaMalloc/cudaFree and no allocating library routine.
//
// Limits and rules:
//   - at most BP_NOALLOC_MAX_ROWS matrix rows (events length) for transpose=1; larger
//     requests are rejected with BP_ENOMEM before anything is enqueued;
//   - the array is shared by every call on a device and keeps the last call's contents;
//     the call resets the active-row counter itself before use;
//   - calls whose work overlaps on the GPU (different streams without ordering, or
//     several host threads) race on the shared array: order them on one stream;
//   - the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call before any
//     stream capture begins.
#include <mutex>

#include "common.cuh"

#define BP_NOALLOC_MAX_ROWS (1 << 21)

namespace bp {

bp_status event_csrmv_transpose_on_scratch(const float* data, bool homo, const void* indices, const void* indptr,
                                           bp_itype itype, int64_t nnz, const void* events, bp_etype et,
                                           int64_t m, int64_t n, float* out, int32_t* list, int32_t* count,
                                           cudaStream_t st);

namespace {

constexpr size_t kHeaderBytes = 256;  // holds the int32 active-row count
constexpr size_t kScratchBytes = kHeaderBytes + sizeof(int32_t) * (size_t)BP_NOALLOC_MAX_ROWS;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch for the current device (looked up once per device).
bp_status scratch_address(void** out) {
  int dev = 0;
  BP_CUDA_TRY(cudaGetDevice(&dev));
  BP_REQUIRE(dev >= 0 && dev < kMaxDevices, BP_ENOTSUP, "event_csrmv_noalloc: device %d beyond %d", dev,
             kMaxDevices);
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_addr[dev] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error("event_csrmv_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev, cudaGetErrorString(e));
      return BP_ECUDA;
    }
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return BP_OK;
}

}  // namespace
}  // namespace bp

using namespace bp;

extern "C" {

int64_t bp_event_csrmv_noalloc_max_rows(void) { return (int64_t)BP_NOALLOC_MAX_ROWS; }

bp_status bp_event_csrmv_noalloc(const float* data, int64_t ndata, const void* indices, const void* indptr,
                                 bp_itype itype, int64_t nnz, const void* events, bp_etype etype, int64_t m,
                                 int64_t n, int32_t transpose, float* out, bp_stream_t stream) {
  clear_error();
  cudaStream_t st = as_cuda(stream);
  BP_REQUIRE(m >= 0 && n >= 0 && nnz >= 0, BP_EINVAL, "event_csrmv_noalloc: negative size m=%lld n=%lld nnz=%lld",
             (long long)m, (long long)n, (long long)nnz);
  BP_REQUIRE(m <= INT32_MAX && n <= INT32_MAX, BP_ENOTSUP, "event_csrmv_noalloc: dimensions beyond int32 range");
  BP_REQUIRE(itype == BP_I32 || itype == BP_I64, BP_EDTYPE, "event_csrmv_noalloc: bad index type %d", (int)itype);
  BP_REQUIRE(etype >= BP_EV_BOOL && etype <= BP_EV_F32_NZ, BP_EDTYPE, "event_csrmv_noalloc: bad event type %d",
             (int)etype);
  BP_REQUIRE(ndata == 1 || ndata == nnz, BP_ESHAPE,
             "event_csrmv_noalloc: the size of data should be 1 or be consistent with indices (%lld vs %lld)",
             (long long)ndata, (long long)nnz);
  if (transpose)
    BP_REQUIRE(m <= (int64_t)BP_NOALLOC_MAX_ROWS, BP_ENOMEM,
               "event_csrmv_noalloc: %lld rows exceed the built-in scratch limit of %d rows "
               "(use bp_event_csrmv with a caller-provided workspace)",
               (long long)m, (int)BP_NOALLOC_MAX_ROWS);
  const int64_t n_out = transpose ? n : m;
  if (n_out == 0) return BP_OK;
  BP_REQUIRE(out != nullptr, BP_EINVAL, "event_csrmv_noalloc: null out");
  if (m == 0 || nnz == 0) {
    BP_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n_out, st));
    return BP_OK;
  }
  BP_REQUIRE(data && indices && indptr && events, BP_EINVAL,
             "event_csrmv_noalloc: null data/indices/indptr/events");
  if (!transpose)  // the gather form needs no scratch
    return bp_event_csrmv(data, ndata, indices, indptr, itype, nnz, events, etype, m, n, 0, out, nullptr, 0, stream);
  void* base = nullptr;
  bp_status s = scratch_address(&base);
  if (s != BP_OK) return s;
  int32_t* count = static_cast<int32_t*>(base);
  int32_t* list = reinterpret_cast<int32_t*>(static_cast<unsigned char*>(base) + kHeaderBytes);
  return event_csrmv_transpose_on_scratch(data, ndata == 1, indices, indptr, itype, nnz, events, etype, m, n, out,
                                          list, count, st);
}

}  // extern "C"
