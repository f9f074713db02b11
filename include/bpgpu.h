/*
 * bpgpu.h -- C ABI of the GB300 (sm_103a) event-driven synaptic propagation
 * library (libbpgpu.so).
 *
 * Conventions for every entry point:
 *   - all array arguments are DEVICE pointers unless stated otherwise;
 *   - work is enqueued on `stream`; no entry point synchronises the stream or
 *     allocates device memory (scratch comes in through `workspace`);
 *   - the return value is a bp_status; BP_OK means the work was enqueued;
 *     bp_last_error() gives a message for the calling thread's last failure;
 *   - outputs are fully overwritten (they need not be zeroed by the caller).
 *
 * The reference binds each operator as a legacy XLA custom call,
 *   void target(cudaStream_t, void** buffers, const char* opaque, size_t len),
 * with all validation done in Python before lowering.  The entry points below
 * take the same operands as typed pointers plus the sizes that the reference
 * packs into `opaque`, and validate them again on the host.
 */
#ifndef BPGPU_H_
#define BPGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* bp_stream_t; /* == cudaStream_t */

typedef enum {
  BP_OK = 0,
  BP_EINVAL = 1,   /* bad argument (null pointer, negative size, bad flag) */
  BP_ESHAPE = 2,   /* inconsistent shapes */
  BP_EDTYPE = 3,   /* unsupported element type */
  BP_ENOMEM = 4,   /* workspace / buffer too small */
  BP_ETIMEOUT = 5, /* a bounded device-side wait gave up */
  BP_ECUDA = 6,    /* CUDA runtime error */
  BP_ENOTSUP = 7   /* valid request that this build does not implement */
} bp_status;

/* index type of CSR `indices` / `indptr` */
typedef enum { BP_I32 = 0, BP_I64 = 1 } bp_itype;

/* event vector type and the truth test applied to it:
 *   BP_EV_BOOL     uint8 (bool) events, event = (e != 0)
 *   BP_EV_F32_POS  float32 events, event = (e > 0)   -- Numba CPU kernels,
 *                  brainpy/_src/math/event/_csr_matvec.py:343-361
 *   BP_EV_F32_NZ   float32 events, event = (e != 0)  -- Taichi kernels,
 *                  brainpy/_src/math/event/_csr_matvec_taichi.py:176-191 */
typedef enum { BP_EV_BOOL = 0, BP_EV_F32_POS = 1, BP_EV_F32_NZ = 2 } bp_etype;

const char* bp_status_string(bp_status s);
const char* bp_last_error(void);
/* library version, e.g. 0x000100 */
int32_t bp_version(void);

/* ---------------------------------------------------------------------------
 * event.info -- spike compaction.
 * Replaces the `event_info` custom call, brainpy/_src/math/event/_info_collection.py:24-43
 * (Numba CPU kernel :144-155, brainpylib GPU target bound at :78-100).
 * ids[0:num] = ascending indices i with event(events[i]); ids[num:n] = -1; num_out[0] = num.
 * ------------------------------------------------------------------------- */
size_t bp_event_info_workspace_size(int64_t n);
bp_status bp_event_info(const void* events, bp_etype etype, int64_t n, int32_t* ids, int32_t* num_out,
                        void* workspace, size_t workspace_bytes, bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * event.csrmv -- product of a CSR matrix (shape m x n) and an event vector.
 * Replaces the custom-call family event_csrmv{_homo,_heter}_float{_int,_long}{_bool,}{_transpose,}
 * bound at brainpy/_src/math/event/_csr_matvec.py:453-500 (Python front-end :38-110) and the
 * Taichi twin csrmv_taichi, brainpy/_src/math/event/_csr_matvec_taichi.py:344-452.
 *   transpose=1: out (n)  out[j] = sum_{i: event(events[i])} A[i, j]       (events length m)
 *   transpose=0: out (m)  out[i] = sum_{j in row i, event(events[j])} A[i,j] (events length n)
 * data: float32, ndata == 1 (homogeneous weight) or ndata == nnz (heterogeneous).
 * Only the truth value of an event is used, never its magnitude (as in the reference).
 * Homogeneous weight with any event type: exact integer event counts, out = (float)count * w.
 * ------------------------------------------------------------------------- */
size_t bp_event_csrmv_workspace_size(int64_t m, int64_t n, int32_t transpose);
bp_status bp_event_csrmv(const float* data, int64_t ndata, const void* indices, const void* indptr,
                         bp_itype itype, int64_t nnz, const void* events, bp_etype etype, int64_t m,
                         int64_t n, int32_t transpose, float* out, void* workspace,
                         size_t workspace_bytes, bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * Column-tiled CSR plan (no counterpart in the reference; it plays the role of a
 * cuSPARSE-style analysis step).  A one-time re-layout of a CSR matrix that the tiled
 * event kernels stream: every row's indices regrouped by column tile of tile_w columns,
 * stored as tile-local uint16 and padded to 8-byte chunks, weights permuted along.
 * The caller owns the device memory (bp_csr_plan_bytes) and keeps it, together with the
 * filled-in bp_csr_plan, for as long as it uses the plan.  A plan is a function of
 * (indices, indptr[, data]) at build time; rebuild it when they change.
 * ------------------------------------------------------------------------- */
typedef struct {
  int64_t m, n, nnz;  /* matrix shape and number of stored entries */
  int32_t tile_w;     /* columns per tile (<= 65535) */
  int32_t n_tiles;    /* ceil(n / tile_w) */
  int32_t heter;      /* 1: the plan carries permuted float32 weights */
  int32_t reserved;
  uint64_t entries;   /* capacity of the padded index array */
  void* mem;          /* device memory holding the plan (caller-owned) */
  size_t bytes;       /* size of mem */
} bp_csr_plan;

/* tile width the tiled kernels run best with on the current device for n columns and
 * clusters of `cluster` CTAs (1, 2, 4 or 8); 0 on error. */
int32_t bp_csr_plan_default_tile(int64_t n, int32_t cluster);
size_t bp_csr_plan_bytes(int64_t m, int64_t n, int64_t nnz, int32_t heter, int32_t tile_w);
/* Builds the plan on `stream` (heterogeneous when ndata == nnz > 1, homogeneous when
 * data is NULL or ndata == 1). */
bp_status bp_csr_plan_build(const float* data, int64_t ndata, const void* indices, const void* indptr,
                            bp_itype itype, int64_t nnz, int64_t m, int64_t n, int32_t tile_w, void* mem,
                            size_t bytes, bp_csr_plan* plan_out, bp_stream_t stream);

/* event.csrmv, transpose=1, on a plan: out (n) = sum of the active rows.  `w_homo` is the
 * homogeneous weight (device pointer to one float) for homogeneous plans and is ignored for
 * heterogeneous ones.  `cluster` = CTAs per column tile (1, 2, 4, 8; 0 = default).
 * Homogeneous: exact integer counts, out = (float)count * w. */
size_t bp_event_csrmv_planned_workspace_size(const bp_csr_plan* plan);
bp_status bp_event_csrmv_planned(const bp_csr_plan* plan, const float* w_homo, const void* events, bp_etype etype,
                                 float* out, int32_t cluster, void* workspace, size_t workspace_bytes,
                                 bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * event.csrmv with no allocation anywhere (no counterpart in the reference).
 * For callers that can pass nothing but operands and the result buffer -- e.g. a legacy
 * XLA custom-call target, which gets its buffers from XLA and has no scratch allocator,
 * and must not cudaMalloc (that would synchronise the device mid-stream).  Same
 * arguments and results as bp_event_csrmv minus the workspace.  The scratch of the
 * transpose path is a fixed __device__ array inside the library, held by every GPU that
 * loads it until exit, sized for at most bp_event_csrmv_noalloc_max_rows() rows (larger
 * m with transpose=1 returns BP_ENOMEM).  All calls on a device share that array: calls
 * whose GPU work overlaps race, so order them on one stream.  The first call on each
 * device looks the array up (cudaGetSymbolAddress); make it before any stream capture.
 * ------------------------------------------------------------------------- */
int64_t bp_event_csrmv_noalloc_max_rows(void);
bp_status bp_event_csrmv_noalloc(const float* data, int64_t ndata, const void* indices, const void* indptr,
                                 bp_itype itype, int64_t nnz, const void* events, bp_etype etype, int64_t m,
                                 int64_t n, int32_t transpose, float* out, bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * Kernel timing (benchmark support; no reference counterpart).
 * When enabled, each operator's dominant kernel launch is bracketed by CUDA events on its
 * stream; bp_timer_collect synchronises them and returns the summed time and launch count,
 * then resets.  Disabled by default; enabling/disabling resets the record.
 * ------------------------------------------------------------------------- */
void bp_timer_enable(int32_t on);
bp_status bp_timer_collect(double* total_ms, int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif /* BPGPU_H_ */
