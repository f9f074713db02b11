/*
 * oracle.h -- CPU restatement of BrainPy's event-driven synaptic propagation
 * path, used ONLY as test infrastructure (the parity reference and the timed CPU
 * baseline).  Nothing in the brainpy_gb300 package links or calls this code.
 *
 * Each function cites the reference file:line it restates (paths relative to
 * the BrainPy source tree).  Float32 "reference-order" outputs follow the
 * reference loop order; FP64 outputs give the exact sums plus the sum of
 * |terms| used to scale tolerances.
 */
#ifndef BP_ORACLE_H_
#define BP_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- LFSR88 (brainpy/_src/math/tifunc.py:48-180) ---- */
void orc_lfsr88_key(uint32_t seed, uint32_t key[4]);
void orc_lfsr88_next_key(uint32_t key[4]);
int32_t orc_lfsr88_random_integers(uint32_t key[4], int32_t low, int32_t high);
float orc_lfsr88_uniform(uint32_t key[4], float low, float high);
float orc_lfsr88_normal(uint32_t key[4], float mu, float sigma);
/* n successive (k0^k1^k2) outputs of the stream seeded with `seed` */
void orc_lfsr88_stream(uint32_t seed, int32_t n, uint32_t* out);

/* ---- just-in-time connectivity ----
 * kind: 0 homo (p0 = weight), 1 uniform (p0 = w_low, p1 = w_high), 2 normal (p0 = mu, p1 = sigma)
 * variant: 0 = Taichi GPU algorithm (brainpy/_src/math/jitconn/_event_matvec_taichi.py:96-155),
 *          1 = Taichi CPU algorithm (_event_matvec_taichi.py:38-85)
 * num_row = output length, num_col = input-vector length (the kernels' own view,
 * after _general_checking reverses `shape` for transpose, _matvec_taichi.py:174-207).
 * Returns the number of connections; if rows/cols/w are non-NULL, the first `cap`
 * connections are written in generation order. */
int64_t orc_jitconn_connections(int32_t kind, float p0, float p1, int32_t clen, uint32_t seed,
                                int64_t num_row, int64_t num_col, int32_t outdim_parallel,
                                int32_t variant, int64_t cap, int64_t* rows, int64_t* cols, float* w);

/* y = M v for the jitconn operators.
 * vec_kind: 0 = bool events (uint8), 1 = float32 events, 2 = dense float32 vector (mv_prob_*).
 * Event semantics follow the chosen variant's kernels (see oracle.c).
 * abs64 is the tolerance scale: sum of |w * v| over the connections, with |w| replaced by
 * |mu| + |w - mu| for normal weights (the magnitude of the operands of mu + sigma*z). */
void orc_jitconn_mv(int32_t kind, int32_t vec_kind, const void* vec, int64_t num_row, int64_t num_col,
                    float p0, float p1, int32_t clen, uint32_t seed, int32_t outdim_parallel,
                    int32_t variant, double* out64, double* abs64);

/* As orc_jitconn_mv with outdim_parallel = 1, computing only the rows flagged in row_mask
 * (num_row bytes); the other rows of out64/abs64 are zero. */
void orc_jitconn_mv_rows(int32_t kind, int32_t vec_kind, const void* vec, int64_t num_row, int64_t num_col,
                         float p0, float p1, int32_t clen, uint32_t seed, int32_t variant,
                         const uint8_t* row_mask, double* out64, double* abs64);

/* ---- event CSR (brainpy/_src/math/event/_csr_matvec.py:321-412) ----
 * ev_kind: 0 = bool (uint8), 1 = float32 with `> 0` (Numba), 2 = float32 with `!= 0` (Taichi)
 * idx64: indices/indptr are int64 when 1, int32 when 0.
 * out32: float32 result in the reference loop order (may be NULL).
 * count32: homogeneous weight only: (float)count * w, the order-free form (may be NULL). */
void orc_event_csrmv(const float* data, int64_t ndata, const void* indices, const void* indptr,
                     int32_t idx64, const void* events, int32_t ev_kind, int64_t m, int64_t n,
                     int32_t transpose, double* out64, double* abs64, float* out32, float* count32);

/* ---- sparse CSR (brainpy/_src/math/sparse/_csr_mv.py:126-164) ---- */
void orc_csrmv(const float* data, int64_t ndata, const void* indices, const void* indptr,
               int32_t idx64, const float* vec, int64_t m, int64_t n, int32_t transpose,
               double* out64, double* abs64, float* out32);

/* ---- event.info (brainpy/_src/math/event/_info_collection.py:144-155) ---- */
int64_t orc_event_info(const uint8_t* events, int64_t n, int32_t* ids);

/* plasticity (brainpy/_src/dnn/linear.py:650-698) and csr2csc (connect/base.py:645-726) */
void orc_csr_on_pre_update(const float* w, const void* indices, const void* indptr, int32_t idx64,
                           int64_t m, const uint8_t* spike, const float* trace, float w_min, float w_max,
                           int64_t nnz, float* out);
void orc_csc_on_post_update(const float* w, const void* pre_ids, const void* indptr, const void* w_ids,
                            int32_t idx64, int64_t n, const uint8_t* spike, const float* trace, float w_min,
                            float w_max, int64_t nnz, float* out);
int64_t orc_fixed_prob_row(uint64_t seed, int64_t row, int64_t n, int32_t K, int32_t multi, int32_t drop_self,
                           int32_t* out);
void orc_csr2csc(const void* indices, const void* indptr, int32_t idx64, int64_t m, int64_t n,
                 int64_t* pre_ids, int64_t* c_indptr, int64_t* w_ids);

/* ---- LIF / Expon / COBA step ----
 * One exponential-Euler step of a population of LifRefLTC (ltc=1) or LifRef (ltc=0)
 * neurons with two Expon+COBA conductance channels (excitatory g_e, inhibitory g_i):
 *   brainpy/_src/dyn/synapses/abstract_models.py:121-134 (Expon),
 *   brainpy/_src/dyn/outs/outputs.py:53-54 (COBA),
 *   brainpy/_src/dyn/neurons/lif.py:461-500 (LifRefLTC.update), :550-556 (LifRef),
 *   brainpy/_src/integrators/ode/exponential.py:354-362 (exp-Euler),
 *   brainpy/_src/math/others.py:94-103 (exprel).
 * dge/dgi: conductance increments from this step's propagation (may be NULL).
 * precise=0: float32 in the reference's operation order; precise=1: float64 arithmetic. */
typedef struct {
  float V_rest, V_th, V_reset, tau, tau_ref, R;
  float tau_e, tau_i, E_e, E_i;
  float input;
  int32_t ltc;
} orc_lif_params;

void orc_lif_step(const orc_lif_params* p, int64_t n, float* V, float* ge, float* gi,
                  float* t_last, uint8_t* spike, const float* dge, const float* dgi,
                  int32_t step_i, float dt, int32_t precise);

/* ---- E/I COBA network (examples/dynamics_simulation/COBA.py:58-109 semantics) ----
 * Neurons [0, n_exc) are excitatory, [n_exc, n) inhibitory, one shared parameter set.
 * exc_* : CSR with n_exc rows over all n posts (E2E and E2I merged), weight we -> g_e
 * inh_* : CSR with n - n_exc rows over all n posts (I2E and I2I merged), weight wi -> g_i
 * Runs `steps` steps starting from the given state; spike counts per step are written to
 * spike_counts (length steps, may be NULL); V trace of the first `trace_steps` steps to
 * v_trace (trace_steps x n, may be NULL).  Propagation uses the order-free count form
 * (Delta g = (float)count * w) when count_mode=1, the reference's sequential float32 adds
 * when count_mode=0. */
void orc_coba_net_run(const orc_lif_params* p, int64_t n, int64_t n_exc,
                      const int32_t* exc_indptr, const int32_t* exc_indices, float we,
                      const int32_t* inh_indptr, const int32_t* inh_indices, float wi,
                      float* V, float* ge, float* gi, float* t_last, uint8_t* spike,
                      int32_t step0, int32_t steps, float dt, int32_t count_mode,
                      int64_t* spike_counts, int32_t trace_steps, float* v_trace);

/* ---- restated reference CPU loops, timed as the CPU baseline (cpu_ref.c) ----
 * brainpy/_src/math/event/_csr_matvec.py:321-339 (transpose, serial, fastmath)
 * brainpy/_src/math/event/_csr_matvec.py:363-386 (non-transpose, prange over rows) */
void cpu_event_csrmv_bool(const float* data, int64_t ndata, const int32_t* indices,
                          const int32_t* indptr, const uint8_t* events, int64_t m, int64_t n,
                          int32_t transpose, float* out);
int32_t cpu_event_csrmv_bool_t_batch(const float* data, int64_t ndata, const int32_t* indices,
                                     const int32_t* indptr, const uint8_t* events, int64_t nb, int64_t m,
                                     int64_t n, float* out);
int32_t cpu_num_threads(void);

void orc_coba_net_run_delayed(const orc_lif_params* p, int64_t n, int64_t n_exc,
                              const int32_t* exc_indptr, const int32_t* exc_indices, float we,
                              const int32_t* inh_indptr, const int32_t* inh_indices, float wi,
                              float* V, float* ge, float* gi, float* t_last, uint8_t* spike,
                              int32_t step0, int32_t steps, float dt, int32_t d_e, int32_t d_i,
                              int32_t L, uint8_t* ring, int64_t* spike_counts);
float orc_bp_expf(float x);
float orc_bp_exprel(float x);

#ifdef __cplusplus
}
#endif
#endif /* BP_ORACLE_H_ */
