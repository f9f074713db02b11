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
  BP_ENOTSUP = 7   /* valid request that this library does not implement */
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
 * sparse.csrmv -- product of a CSR matrix and a dense float32 vector.
 * Replaces gpu_sparse.cuda_csr_matvec (cuSPARSE; brainpy/_src/math/sparse/_csr_mv.py:197-208),
 * the brainpylib csrmv_{homo,heter}_{scalar,vector} targets (:257-396) and the Taichi twin
 * csrmv_taichi (brainpy/_src/math/sparse/_csr_mv_taichi.py:28-287).
 *   transpose=1: out (n) = A^T vec (vec length m);  transpose=0: out (m) = A vec (vec length n).
 * Homogeneous weight (ndata == 1): vector values are summed and multiplied by w once.
 * ------------------------------------------------------------------------- */
bp_status bp_csrmv(const float* data, int64_t ndata, const void* indices, const void* indptr, bp_itype itype,
                   int64_t nnz, const float* vec, int64_t m, int64_t n, int32_t transpose, float* out,
                   bp_stream_t stream);

/* Weight cotangent of event.csrmv / sparse.csrmv (the heterogeneous-data branch of their
 * transpose rules, brainpy/_src/math/event/_csr_matvec.py:545-547 and
 * brainpy/_src/math/sparse/_csr_mv.py:237-239, which build COO rows and gather):
 *   out[j] = x[i] * y[indices[j]]  for every stored entry j of row i (nnz outputs),
 * 0 where indices[j] is outside [0, n) or j lies outside every row.  For transpose=1,
 * x = events or vector (length m) and y = cotangent (length n); for transpose=0 the roles swap
 * (x = cotangent, y = vector). */
bp_status bp_csr_sampled_outer(const float* x, const float* y, const void* indices, const void* indptr,
                               bp_itype itype, int64_t nnz, int64_t m, int64_t n, float* out, bp_stream_t stream);

/* STDP weight updates of the CSR layers (brainpy/_src/dnn/linear.py:650-698, the numba targets
 * _cpu_csr_on_pre_update / _cpu_csc_on_pre_update behind csr_on_pre_update and
 * csc_on_post_update, called from _CSRLayer.stdp_update :517-543).
 *   on_pre:  for every row i with spike[i] (bool, or float != 0) and every synapse k of row i,
 *            w[k] = min(max(w[k] + trace[indices[k]], w_min), w_max)   (trace: length n)
 *   on_post: for every column i with spike[i] and every CSC entry k of column i,
 *            w[w_ids[k]] = min(max(w[w_ids[k]] + trace[pre_ids[k]], w_min), w_max)   (trace: length m)
 * (pre_ids, indptr, w_ids) is the CSC form of csr2csc (connect/base.py:645-726), n columns,
 * m rows.  w_out receives the result; w_out == w_in updates in place (event-driven: only the
 * spiking rows are touched), otherwise w_in is copied first, as the reference returns a new
 * array.  NaN propagates through the clip as in numpy.  Workspace: bp_stdp_workspace_size(m)
 * bytes for on_pre, bp_stdp_workspace_size(n) for on_post (the compacted spike list). */
size_t bp_stdp_workspace_size(int64_t rows);
bp_status bp_csr_on_pre_update(const float* w_in, float* w_out, const void* indices, const void* indptr,
                               bp_itype itype, int64_t nnz, int64_t m, int64_t n, const void* spike, bp_etype etype,
                               const float* trace, float w_min, float w_max, void* workspace, size_t workspace_bytes,
                               bp_stream_t stream);
bp_status bp_csc_on_post_update(const float* w_in, float* w_out, const void* pre_ids, const void* indptr,
                                const void* w_ids, bp_itype itype, int64_t nnz, int64_t n, int64_t m,
                                const void* spike, bp_etype etype, const float* trace, float w_min, float w_max,
                                void* workspace, size_t workspace_bytes, bp_stream_t stream);

/* FixedProb connectivity built on the device (replaces the numba loop of
 * brainpy/_src/connect/random_conn.py:73-128, FixedProb._iii / build_csr).  Row r (rows with
 * row_mask[r] == 0 are empty; row_mask may be NULL) takes K = int(n * prob) columns: the first K
 * distinct values of a counter-based i.i.d. uniform sequence on [0, n) seeded by (seed, r) -- a
 * uniformly random K-subset in random order, the law of rng.choice(n, K, replace=False) -- or,
 * with allow_multi, the first K values (with repeats).  include_self == 0 (m == n only) removes
 * the diagonal entries drawn, as the reference does after drawing.  K <= 16384 without
 * allow_multi.
 *   bp_fixed_prob_row_lengths: lengths[r] (int32; -1 flags a row whose generation overran its
 *     draw bound, which does not happen for valid arguments).
 *   bp_fixed_prob_fill: indices[indptr[r] .. indptr[r+1]) for every row (int32 columns), with
 *     indptr the exclusive sum of the lengths (K * r when include_self and no mask). */
bp_status bp_fixed_prob_row_lengths(int64_t m, int64_t n, int32_t K, uint64_t seed, int32_t allow_multi,
                                    int32_t include_self, const uint8_t* row_mask, int32_t* lengths,
                                    bp_stream_t stream);
bp_status bp_fixed_prob_fill(int64_t m, int64_t n, int32_t K, uint64_t seed, int32_t allow_multi,
                             int32_t include_self, const uint8_t* row_mask, const int64_t* indptr, int32_t* indices,
                             bp_stream_t stream);

/* CSR utilities (brainpy/_src/math/sparse/_utils.py:44-114): COO row ids of every stored entry
 * (same index type as indptr), and the dense (m x n, row-major) matrix with duplicates added. */
bp_status bp_csr_to_coo(const void* indptr, bp_itype itype, int64_t m, int64_t nnz, void* rows, bp_stream_t stream);
bp_status bp_csr_to_dense(const float* data, int64_t ndata, const void* indices, const void* indptr, bp_itype itype,
                          int64_t nnz, int64_t m, int64_t n, float* dense, bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * Just-in-time connectivity: y = M v with M regenerated from LFSR88 streams.
 * Replaces the custom-call families gpu_jit_event_csrmv_{,atomic_}prob_{homo,uniform,normal}_v2*
 * (brainpy/_src/math/jitconn/_event_matvec.py:198-229, :384-414, :578-608) and
 * gpu_jit_csrmv_{,atomic_}prob_*_v2* (_matvec.py:341-378, :535-574, :717-760), whose source is
 * not public; the connectivity follows the reference's in-tree Taichi kernels bit for bit:
 *   BP_JC_TAICHI_GPU: _event_matvec_taichi.py:96-155 and twins (32 lane streams per owner),
 *   BP_JC_TAICHI_CPU: _event_matvec_taichi.py:38-85 and twins (one stream per owner).
 * num_row = output length, num_col = input length (the kernels' own view: for transpose=True
 * the front-end passes shape[1] outputs and shape[0] inputs).  kind: p0/p1 = weight/unused,
 * w_low/w_high or mu/sigma.  clen = the connection length int(ceil(1/p))*2-1; seed as uint32.
 * outdim_parallel=1: pull (deterministic warp sum per output row); 0: push (atomic adds).
 * Event vectors: only whether an entry is nonzero matters, except that the GPU pull kernels
 * multiply a float32 event value in (as the reference's GPU kernels do).
 * ------------------------------------------------------------------------- */
typedef enum { BP_JC_HOMO = 0, BP_JC_UNIFORM = 1, BP_JC_NORMAL = 2 } bp_jc_kind;
typedef enum { BP_VEC_EVENT_BOOL = 0, BP_VEC_EVENT_F32 = 1, BP_VEC_DENSE_F32 = 2 } bp_jc_vec;
typedef enum { BP_JC_TAICHI_GPU = 0, BP_JC_TAICHI_CPU = 1 } bp_jc_variant;

bp_status bp_jitconn_mv(bp_jc_kind kind, bp_jc_vec vec_kind, const void* vec, int64_t num_col, int64_t num_row,
                        float p0, float p1, int32_t clen, uint32_t seed, int32_t outdim_parallel,
                        bp_jc_variant variant, float* out, bp_stream_t stream);
/* Writes M densely (row-major num_row x num_col float32, zeros elsewhere); every connection is
 * generated once, so this is the exact connectivity and weights the mv kernels use. */
bp_status bp_jitconn_dense(bp_jc_kind kind, float p0, float p1, int32_t clen, uint32_t seed, int64_t num_row,
                           int64_t num_col, int32_t outdim_parallel, bp_jc_variant variant, float* dense,
                           bp_stream_t stream);
/* The pull connectivity (Taichi GPU algorithm, outdim_parallel=1) of one projection with
 * num_row outputs and num_col inputs, stored by input: for input column c, the output rows
 * whose streams visit c.  Pass 0 writes counts[c] (num_col uint32: the column's rows).  Pass 1
 * writes row + row_offset at indices[base[c] .. base[c] + counts[c]) (base: num_col int64,
 * indices: BP_I32 or BP_I64, nnz entries; positions outside [0, nnz) are skipped), in no fixed
 * order inside a column.  With the counts as row lengths this is the presynaptic-row CSR of the
 * projection, the same connections the jitconn mv kernels generate on every call (replaces
 * regenerating them: brainpy/_src/math/jitconn/_event_matvec_taichi.py:96-155 walks these
 * streams per call). */
bp_status bp_jitconn_csr(int32_t pass, int32_t clen, uint32_t seed, int64_t num_row, int64_t num_col,
                         uint32_t* counts, const int64_t* base, int64_t row_offset, void* indices, int64_t nnz,
                         bp_itype itype, bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * Column-tiled CSR plan (no counterpart in the reference; it plays the role of a
 * cuSPARSE-style analysis step).  A one-time re-layout of a CSR matrix that the tiled
 * event kernels stream: every row's indices regrouped by column tile of tile_w columns,
 * stored as tile-local uint16 and padded to 16-byte chunks (8 entries), weights permuted
 * along.  Plans hold fewer than 2^32 chunks (about 3.4e10 entries).
 * The caller owns the device memory (bp_csr_plan_bytes) and keeps it, together with the
 * filled-in bp_csr_plan, for as long as it uses the plan.  A plan is a function of
 * (indices, indptr[, data]) at build time; rebuild it when they change.
 * ------------------------------------------------------------------------- */
typedef struct {
  int64_t m, n, nnz;  /* matrix shape and number of stored entries */
  int32_t tile_w;     /* columns per tile (<= 65535) */
  int32_t n_tiles;    /* ceil(n / tile_w) */
  int32_t heter;      /* 1: the plan carries permuted float32 weights */
  int32_t variant;    /* tiled-kernel variant G | RND << 8 | PF << 16 (lanes per segment, chunk rounds,
                         L1 prefetch of a segment's extra chunks), 0 = chosen from the mean segment length; set by the caller,
                         e.g. after timing the candidates of bp_csr_plan_variants */
  uint64_t entries;   /* capacity of the padded index array */
  void* mem;          /* device memory holding the plan (caller-owned) */
  size_t bytes;       /* size of mem */
  int32_t kind;       /* 0: general plan (cluster kernels; every product, batches, weights);
                         1: counting plan (split kernels; homogeneous weight, one event vector a
                         call; tile_w from bp_csr_plan_count_tile).  bp_csr_plan_build sets 0; the
                         caller sets 1 on a homogeneous plan built with a counting tile;
                         2: fixed-weight plan (set by bp_csr_plan_fix_weights). */
} bp_csr_plan;

/* tile width the tiled kernels run best with on the current device for n columns and
 * clusters of `cluster` CTAs (1, 2, 4 or 8); 0 on error. */
int32_t bp_csr_plan_default_tile(int64_t n, int32_t cluster);
/* tile width of a counting plan for n columns, 0 when n is too small for one (n < 2^19).
 * A counting plan (bp_csr_plan.kind = 1) has tiles as wide as one CTA's shared memory holds
 * 16-bit counters packed in pairs (up to 65,472 columns).  bp_event_csrmv_planned runs it with
 * R CTAs per tile (R = SMs / n_tiles, at most 16), each counting its share of the active rows,
 * and a second kernel that adds the R partial counts of every column (the workspace holds
 * them).  A call reads half as many, twice as long segments as with the default tile (DRAM
 * serves random reads of up to ~128 bytes at a fixed rate), at the cost of the partial counts'
 * round trip through the workspace; which is faster depends on the matrix and the rate, so
 * it is a candidate for timing rather than a default.  Counting plans serve homogeneous
 * weights and single event vectors (BP_ENOTSUP for dense vectors and batches). */
int32_t bp_csr_plan_count_tile(int64_t n);
size_t bp_csr_plan_bytes(int64_t m, int64_t n, int64_t nnz, int32_t heter, int32_t tile_w);
/* The compiled tiled-kernel variants (bp_csr_plan.variant codes): writes up to `cap` codes into
 * `codes` and returns how many there are. */
int32_t bp_csr_plan_variants(int32_t* codes, int32_t cap);
/* Builds the plan on `stream` (heterogeneous when ndata == nnz > 1, homogeneous when
 * data is NULL or ndata == 1). */
bp_status bp_csr_plan_build(const float* data, int64_t ndata, const void* indices, const void* indptr,
                            bp_itype itype, int64_t nnz, int64_t m, int64_t n, int32_t tile_w, void* mem,
                            size_t bytes, bp_csr_plan* plan_out, bp_stream_t stream);

/* device arrays inside a plan: seg_off[m][n_tiles+1] (segment t of row r is the 16-byte chunks
 * [seg_off[r][t], seg_off[r][t+1]) of idx, 8 tile-local indices each, padded with the index tile_w),
 * idx[entries], w[entries] or NULL */
bp_status bp_csr_plan_arrays(const bp_csr_plan* plan, const uint32_t** seg_off, const uint16_t** idx,
                             const float** w);

/* Fixed-weight plans (bp_csr_plan.kind = 2; event.csrmv transpose with per-synapse weights, one
 * event vector a call).  bp_csr_plan_fix_weights converts a general heterogeneous plan's weights in
 * place to int32 fixed point q = rint(w * 2^k) (the caller picks k so that no column's sum of |w|
 * times 2^k reaches 2^31) and lists the nonzero weights with |w| < tau as (row, column, w) in
 * side_rows / side_cols / side_w (up to side_cap of them; *side_count, a device word, receives the
 * full count).  With convert = 0 it only counts them.  The caller sorts the listed entries by row
 * and passes the rows that hold any (side_rows[0 .. side_nrows)) with each one's entries at
 * [side_ptr[i], side_ptr[i + 1]) of side_cols / side_w to bp_event_csrmv_planned_fixed, which adds the fixed-
 * point weights with exact integer shared-memory adds (out = (float)sum * 2^-k) and then the listed
 * weights with float atomics.  With tau = 2^-(k+1) / 5e-6 every fixed-point term is within 5e-6
 * of its weight, relative, so a sum stays within 1e-5 of the exact sum of its terms' magnitudes. */
bp_status bp_csr_plan_fix_weights(bp_csr_plan* plan, int32_t k, float tau, int32_t* side_rows, int32_t* side_cols,
                                  float* side_w, int64_t side_cap, uint64_t* side_count, int32_t convert,
                                  bp_stream_t stream);
/* The fixed-weight call reads each chunk as one record, so a segment is one contiguous read:
 * bp_csr_plan_fix_interleave writes them into fx (bp_csr_plan_fix_interleave_bytes(plan,
 * record_bytes) bytes on a 16-byte boundary, kept beside the plan).  record_bytes = 48: the 8
 * indices, then the 8 int32 weights.  record_bytes = 40: the 8 indices, the low 16 bits of the 8
 * weights and their high bytes, for weights in [-2^23, 2^23) (when max |w| * 2^k < 2^23 - 1);
 * the weights outside that range are added to *unfit (a device word, required), and the records
 * are usable only while it stays 0.  Both forms give the same results bit for bit;
 * bp_event_csrmv_planned_fixed takes the record size the chunks were written with. */
size_t bp_csr_plan_fix_interleave_bytes(const bp_csr_plan* plan, int32_t record_bytes);
bp_status bp_csr_plan_fix_interleave(const bp_csr_plan* plan, int32_t record_bytes, void* fx, size_t fx_bytes,
                                     uint64_t* unfit, bp_stream_t stream);
bp_status bp_event_csrmv_planned_fixed(const bp_csr_plan* plan, const void* fx, int32_t record_bytes,
                                       const int32_t* side_rows,
                                       const int32_t* side_ptr, const int32_t* side_cols, const float* side_w,
                                       int64_t side_nrows, const void* events, bp_etype etype, float* out,
                                       int32_t cluster, void* workspace, size_t workspace_bytes,
                                       bp_stream_t stream);

/* event.csrmv, transpose=1, on a plan: out (n) = sum of the active rows.  `w_homo` is the
 * homogeneous weight (device pointer to one float) for homogeneous plans and is ignored for
 * heterogeneous ones.  `cluster` = CTAs per column tile (1, 2, 4, 8; 0 = default).
 * Homogeneous: exact integer counts, out = (float)count * w. */
size_t bp_event_csrmv_planned_workspace_size(const bp_csr_plan* plan);
bp_status bp_event_csrmv_planned(const bp_csr_plan* plan, const float* w_homo, const void* events, bp_etype etype,
                                 float* out, int32_t cluster, void* workspace, size_t workspace_bytes,
                                 bp_stream_t stream);

/* sparse.csrmv, transpose=1, on a plan: out (n) = A^T vec.  Entries with vec[i] == 0 are
 * skipped; `w_homo` as for bp_event_csrmv_planned.  Workspace: bp_event_csrmv_planned_workspace_size. */
bp_status bp_csrmv_planned(const bp_csr_plan* plan, const float* w_homo, const float* vec, float* out,
                           int32_t cluster, void* workspace, size_t workspace_bytes, bp_stream_t stream);

/* sparse.csrmv, transpose=0, on a plan: out (m) = A vec (vec length n).  Each CTA stages one
 * column tile of vec in shared memory and sums its rows' segments for that tile; the per-tile
 * partial sums (workspace: bp_csrmv_planned_n_workspace_size(plan) = 4 * m * n_tiles bytes)
 * are added in tile order.  Homogeneous: w * (sum of the vector entries), as the reference's
 * homogeneous non-transpose kernels apply the weight once (brainpy/_src/math/sparse/
 * _csr_mv_taichi.py:53-65). */
size_t bp_csrmv_planned_n_workspace_size(const bp_csr_plan* plan);
bp_status bp_csrmv_planned_n(const bp_csr_plan* plan, const float* w_homo, const float* vec, float* out,
                             void* workspace, size_t workspace_bytes, bp_stream_t stream);

/* A batch of `batch` vectors (0..65535) through one plan in one launch pair -- the batched form
 * that replaces the reference's batching rule for these primitives, a sequential lax.scan of
 * single calls (brainpy/_src/math/op_register/utils.py:16-38, registered for event.csrmv at
 * brainpy/_src/math/event/_csr_matvec.py:556).  `events` / `vec` hold batch rows of m
 * (contiguous), `out` batch rows of n; row b of out is the single-vector result for row b.
 * Workspace: bp_event_csrmv_planned_batch_workspace_size(plan, batch). */
size_t bp_event_csrmv_planned_batch_workspace_size(const bp_csr_plan* plan, int32_t batch);
bp_status bp_event_csrmv_planned_batch(const bp_csr_plan* plan, const float* w_homo, const void* events,
                                       bp_etype etype, int32_t batch, float* out, int32_t cluster, void* workspace,
                                       size_t workspace_bytes, bp_stream_t stream);
bp_status bp_csrmv_planned_batch(const bp_csr_plan* plan, const float* w_homo, const float* vec, int32_t batch,
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
 * The address is kept per device ordinal for the life of the process: after a
 * cudaDeviceReset (or with another context on the device) it is stale, so do not call this
 * entry point across a device reset.
 * ------------------------------------------------------------------------- */
int64_t bp_event_csrmv_noalloc_max_rows(void);
bp_status bp_event_csrmv_noalloc(const float* data, int64_t ndata, const void* indices, const void* indptr,
                                 bp_itype itype, int64_t nnz, const void* events, bp_etype etype, int64_t m,
                                 int64_t n, int32_t transpose, float* out, bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * LIF / Expon / COBA neurons (the consumer of the propagation operators).
 * No reference counterpart as a kernel: the reference lowers these to XLA elementwise code.
 * Semantics: LifRefLTC (ltc=1) / LifRef (ltc=0), brainpy/_src/dyn/neurons/lif.py:348-556,
 * with an excitatory and an inhibitory Expon conductance (abstract_models.py:24-134) feeding
 * COBA outputs (outputs.py:16-54), exponential Euler (integrators/ode/exponential.py:338-364).
 * Order within a step: g += dg; g decays; V integrates with the decayed g; refractory;
 * threshold; reset.  t = float32(step) * dt.  float32, no contraction: results agree bit for
 * bit with a CPU evaluation in the same operation order.
 * ------------------------------------------------------------------------- */
typedef struct {
  float V_rest, V_th, V_reset, tau, tau_ref, R;
  float tau_e, tau_i, E_e, E_i;
  float input; /* constant external current (the `inp` passed to the neuron update) */
  int32_t ltc; /* 1: LifRefLTC (conductance currents inside the derivative); 0: LifRef */
} bp_lif_params;

/* One step of n neurons: dge/dgi (nullable) are this step's conductance increments. */
bp_status bp_lif_coba_step(const bp_lif_params* params, int64_t n, float* V, float* ge, float* gi, float* t_last,
                           uint8_t* spike, const float* dge, const float* dgi, int32_t step, float dt,
                           bp_stream_t stream);

/* As bp_lif_coba_step with the step index read on the device: step = *step_dev + step_offset
 * (lets one captured CUDA graph of several steps be replayed at any time). */
bp_status bp_lif_coba_step_dev(const bp_lif_params* params, int64_t n, float* V, float* ge, float* gi,
                               float* t_last, uint8_t* spike, const float* dge, const float* dgi,
                               const int32_t* step_dev, int32_t step_offset, float dt, bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * Whole E/I COBA networks in one persistent launch (examples/dynamics_simulation/COBA.py:58-109,
 * run by DSRunner: brainpy/_src/runners.py:619-665).  No reference counterpart as a kernel.
 * A network is n neurons ([0, n_exc) excitatory) with one homogeneous-weight CSR matrix over all
 * n pre-synaptic rows and n post-synaptic columns (E2E+E2I rows, I2E+I2I rows), given as a plan
 * (bp_csr_plan) whose tiles have tile_w <= 4096 columns; the network runs on a thread-block
 * cluster of n_tiles CTAs (n_tiles <= 16), every CTA owning one tile of neurons in shared memory.
 * Per step: the previous step's spikes are propagated (exact integer counts; dg = count * w),
 * then every neuron is updated.  The descriptor array lives in device memory.
 * ------------------------------------------------------------------------- */
typedef struct {
  int32_t n, n_exc;
  int32_t tile_w, n_tiles;
  const uint32_t* seg_off;   /* plan arrays of the network's CSR (bp_csr_plan, homogeneous) */
  const uint16_t* idx;
  float we, wi;
  bp_lif_params p;
  float *V, *ge, *gi, *t_last; /* state, length n, updated in place */
  uint8_t* spike;              /* spikes of the last completed step, length n */
  int32_t* spike_counts;       /* [steps] spikes per step, accumulated into (nullable) */
  uint32_t* raster;            /* [steps][ceil(n/32)] spike bits (nullable) */
  float* v_trace;              /* [trace_steps][n] membrane potential (nullable) */
  int32_t trace_steps;
  int32_t step_limit;          /* > 0: this network stops after step_limit of the launch's steps */
  int32_t step0;               /* time index of this network's first step (added to the launch's step0) */
  /* Synaptic delays (VarDelay, brainpy/_src/delay.py:334-373), in steps (ceil(delay / dt)): at
   * step T the excitatory rows propagate the spikes of step T - delay_e, the inhibitory rows
   * those of T - delay_i (0: the previous step's spikes, i.e. `spike`).  ring holds the spike
   * bits of the last ring_len steps, step T in slot T mod ring_len, [ring_len][ceil(n/32)] words,
   * zero before the first step; ring_len >= max(delay_e, delay_i), <= 64.  ring may be NULL
   * (ring_len 0) when both delays are 0. */
  int32_t delay_e, delay_i;
  int32_t ring_len;
  uint32_t* ring;
} bp_net_desc;

/* The spike history of bp_net_desc for the per-operator path: bp_spike_ring_record stores the
 * n spikes (bytes) of step T as bits in slot T mod ring_len; bp_spike_ring_read writes, for
 * neurons [lo, lo + count), the bits of step T - delay as bytes into out.  T = step, plus
 * *step_dev when step_dev is not NULL (device-side time index for CUDA-graph replay). */
bp_status bp_spike_ring_record(const uint8_t* spike, int64_t n, uint32_t* ring, int32_t ring_len, int64_t step,
                               const int32_t* step_dev, bp_stream_t stream);
bp_status bp_spike_ring_read(const uint32_t* ring, int32_t ring_len, int64_t n, int64_t lo, int64_t count,
                             int32_t delay, int64_t step, const int32_t* step_dev, uint8_t* out, bp_stream_t stream);

/* largest n_tiles (cluster size) bp_net_run accepts, and the tile width it expects */
int32_t bp_net_max_tiles(void);
int32_t bp_net_tile_width(void);
/* Runs `steps` steps (global step indices step0 .. step0+steps-1) of num_nets networks that all
 * have n_tiles == cluster, concurrently (one cluster per network). */
bp_status bp_net_run(const bp_net_desc* descs_device, int32_t num_nets, int32_t cluster, int32_t step0,
                     int32_t steps, float dt, bp_stream_t stream);

/* ---------------------------------------------------------------------------
 * One E/I COBA network larger than a cluster, in one persistent launch over the GPU (the
 * DSRunner loop of examples/dynamics_simulation/COBA.py run by brainpy/_src/runners.py:619-665;
 * no reference counterpart as a kernel).  The network's plan (bp_csr_plan of the merged CSR
 * over all n rows and columns) has tiles of tile_w = bp_net_grid_tile(n) columns; each tile is
 * owned by a cluster of 4 CTAs, every CTA updating a quarter of the tile's neurons.  Each step
 * propagates the previous step's spikes (exact integer counts, excitatory and inhibitory rows
 * counted separately; no column may have 65,536 or more incoming entries), updates the neurons
 * (dg = count * w, the LIF step of bp_lif_coba_step) and lists the new spikes, then waits on a
 * grid-wide barrier whose waits are bounded: a wait that runs out ends the launch early and
 * sets the error word (in the workspace, zeroed by the caller once) that bp_net_grid_error
 * reads.  Synaptic delays work as in bp_net_run (the ring in desc); rasters are not supported
 * (BP_ENOTSUP); desc is a host pointer.
 * ------------------------------------------------------------------------- */
/* tile width for an n-neuron network, 0 when its clusters cannot all be resident at once */
int32_t bp_net_grid_tile(int64_t n);
size_t bp_net_grid_workspace_size(int64_t n, int32_t tile_w);
bp_status bp_net_run_grid(const bp_net_desc* desc, int32_t step0, int32_t steps, float dt, void* workspace,
                          size_t workspace_bytes, bp_stream_t stream);
/* the error word of the runs on this workspace since it was zeroed (0: every barrier wait
 * ended; the caller zeroes a new workspace); synchronises */
bp_status bp_net_grid_error(const void* workspace, int32_t* error, bp_stream_t stream);
/* A just-in-time network in the push form (the four EventJitFPHomoLinear projections with
 * atomic=True, i.e. jitconn.event_mv_prob_homo with outdim_parallel=False, Taichi GPU streams) in
 * one persistent cooperative launch, one CTA per SM: each step regenerates the spiking neurons'
 * connections (seeds: E->E, E->I, I->E, I->I; clen = conn_len(prob)) and adds the weight of every
 * connection with a float atomic, as the per-operator path does, so the results are equal bit for
 * bit.  desc's plan fields are unused; no delays, no raster.  The error word is read by
 * bp_net_grid_error on this workspace. */
size_t bp_net_grid_jit_workspace_size(int64_t n);
bp_status bp_net_run_grid_jit(const bp_net_desc* desc, const uint32_t* seeds, int32_t clen, int32_t step0,
                              int32_t steps, float dt, void* workspace, size_t workspace_bytes, bp_stream_t stream);
/* 1 when the last bp_net_run_grid launched with cooperative scheduling, 0 when the device refused
 * cooperative scheduling together with clusters and the launch went without it (every cluster
 * was checked to be resident at once), -1 before the first launch */
int32_t bp_net_grid_cooperative(void);

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
