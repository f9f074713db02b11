/*
 * oracle.c -- CPU restatement of BrainPy's event-driven synaptic propagation
 * path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of bench.py compare against it; the product path never
 * calls it.
 *
 * Compiled with -O2 -ffp-contract=off (no fast-math) so every float32
 * expression below is evaluated exactly in the order written.
 *
 * Integer semantics of the Taichi kernels: Taichi derives the result type of a
 * mixed binary operation from C++'s own rules (u32 op i32 -> u32), so all the
 * stream arithmetic below is done in uint32_t, including the wrap-around of
 * `step * index - 1` for lane 0.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../brainpy_gb300/csrc/bp_math.h"

/* ------------------------------------------------------------------------ */
/* LFSR88                                                                    */
/* ------------------------------------------------------------------------ */

/* brainpy/_src/math/tifunc.py:47-67: key = (seed+1, seed+7, seed+15, 0) in u32 */
void orc_lfsr88_key(uint32_t seed, uint32_t key[4]) {
  key[0] = seed + 1u;
  key[1] = seed + 7u;
  key[2] = seed + 15u;
  key[3] = 0u;
}

/* brainpy/_src/math/tifunc.py:70-86 (L'Ecuyer's combined Tausworthe generator) */
void orc_lfsr88_next_key(uint32_t key[4]) {
  uint32_t b = ((key[0] << 13) ^ key[0]) >> 19;
  uint32_t s1 = ((key[0] & 4294967294u) << 12) ^ b;
  b = ((key[1] << 2) ^ key[1]) >> 25;
  uint32_t s2 = ((key[1] & 4294967288u) << 4) ^ b;
  b = ((key[2] << 3) ^ key[2]) >> 11;
  uint32_t s3 = ((key[2] & 4294967280u) << 17) ^ b;
  key[0] = s1;
  key[1] = s2;
  key[2] = s3;
  key[3] = b;
}

/* brainpy/_src/math/tifunc.py:136-147: (k0^k1^k2) % (high+1-low) + low, u32 arithmetic,
 * result cast to int32 */
int32_t orc_lfsr88_random_integers(uint32_t key[4], int32_t low, int32_t high) {
  orc_lfsr88_next_key(key);
  uint32_t x = key[0] ^ key[1] ^ key[2];
  uint32_t span = (uint32_t)(high + 1 - low);
  return (int32_t)(x % span + (uint32_t)low);
}

/* brainpy/_src/math/tifunc.py:171-180: f32(k0^k1^k2) * f32(2.3283064365386963e-10) */
static float lfsr88_rand(uint32_t key[4]) {
  orc_lfsr88_next_key(key);
  uint32_t x = key[0] ^ key[1] ^ key[2];
  float u = (float)x;
  return u * 2.3283064365386963e-10f;
}

/* brainpy/_src/math/tifunc.py:156-168: r * (high - low) + low in float32 */
float orc_lfsr88_uniform(uint32_t key[4], float low, float high) {
  float r = lfsr88_rand(key);
  float span = high - low;
  float t = r * span;
  return t + low;
}

/* brainpy/_src/math/tifunc.py:89-133: Box-Muller, sin branch, u1 clamped to 1e-10 */
float orc_lfsr88_normal(uint32_t key[4], float mu, float sigma) {
  float u1 = lfsr88_rand(key);
  float u2 = lfsr88_rand(key);
  if (u1 < 1e-10f) u1 = 1e-10f;
  float lg = logf(u1);
  float mag = sqrtf(-2.0f * lg);
  float ang = 6.28318530717958648f * u2;
  float z = mag * sinf(ang);
  float sz = sigma * z;
  return mu + sz;
}

void orc_lfsr88_stream(uint32_t seed, int32_t n, uint32_t* out) {
  uint32_t key[4];
  orc_lfsr88_key(seed, key);
  for (int32_t i = 0; i < n; ++i) {
    orc_lfsr88_next_key(key);
    out[i] = key[0] ^ key[1] ^ key[2];
  }
}

/* ------------------------------------------------------------------------ */
/* just-in-time connectivity                                                 */
/* ------------------------------------------------------------------------ */

static float draw_weight(int32_t kind, uint32_t key[4], float p0, float p1) {
  if (kind == 1) return orc_lfsr88_uniform(key, p0, p1);
  if (kind == 2) return orc_lfsr88_normal(key, p0, p1);
  return p0;
}

typedef void (*conn_visit)(void* ctx, int64_t row, int64_t col, float w);

/* Walks every connection of the just-in-time matrix in generation order.
 * Only streams whose "owner" index passes `owner_active` are walked: the owner is the
 * output row for outdim_parallel=1 and the input column for outdim_parallel=0 (the
 * push kernels skip inactive columns before drawing anything, so their streams are
 * never consumed; the pull kernels walk every stream). */
static void jitconn_walk(int32_t kind, float p0, float p1, int32_t clen, uint32_t seed,
                         int64_t num_row, int64_t num_col, int32_t outdim_parallel, int32_t variant,
                         const uint8_t* owner_active, conn_visit visit, void* ctx) {
  uint32_t key[4];
  if (variant == 0) {
    /* Taichi GPU algorithm: 32 lane streams per owner.
     * pull: brainpy/_src/math/jitconn/_event_matvec_taichi.py:126-154
     * push: brainpy/_src/math/jitconn/_event_matvec_taichi.py:96-123 */
    int32_t nr = (int32_t)num_row;
    int32_t sh = (nr + 1) >> 5;
    uint32_t step = (uint32_t)(sh > 1 ? sh : 1);
    int64_t n_owner = outdim_parallel ? num_row : num_col;
    uint32_t lim = (uint32_t)(outdim_parallel ? num_col : num_row);
    for (int64_t o = 0; o < n_owner; ++o) {
      if (owner_active && !owner_active[o]) continue;
      for (int32_t lane = 0; lane < 32; ++lane) {
        uint32_t i = (uint32_t)(o * 32 + lane);
        uint32_t c = step * (uint32_t)lane - 1u;
        uint32_t end = c + step;
        if (lim < end) end = lim;
        orc_lfsr88_key(seed + i, key);
        c += (uint32_t)orc_lfsr88_random_integers(key, 1, clen);
        while (c < end) {
          float w = draw_weight(kind, key, p0, p1);
          if (outdim_parallel) visit(ctx, o, (int64_t)c, w);
          else visit(ctx, (int64_t)c, o, w);
          c += (uint32_t)orc_lfsr88_random_integers(key, 1, clen);
        }
      }
    }
  } else {
    /* Taichi CPU algorithm: one stream per owner covering the whole other dimension.
     * pull: brainpy/_src/math/jitconn/_event_matvec_taichi.py:62-85
     * push: brainpy/_src/math/jitconn/_event_matvec_taichi.py:38-59 */
    int64_t n_owner = outdim_parallel ? num_row : num_col;
    int32_t lim = (int32_t)(outdim_parallel ? num_col : num_row);
    for (int64_t o = 0; o < n_owner; ++o) {
      if (owner_active && !owner_active[o]) continue;
      orc_lfsr88_key(seed + (uint32_t)o, key);
      int32_t c = orc_lfsr88_random_integers(key, 0, clen - 1);
      while (c < lim) {
        float w = draw_weight(kind, key, p0, p1);
        if (outdim_parallel) visit(ctx, o, c, w);
        else visit(ctx, c, o, w);
        c += orc_lfsr88_random_integers(key, 1, clen);
      }
    }
  }
}

typedef struct {
  int64_t n, cap;
  int64_t *rows, *cols;
  float* w;
} conn_list;

static void conn_list_visit(void* ctx, int64_t row, int64_t col, float w) {
  conn_list* l = (conn_list*)ctx;
  if (l->n < l->cap) {
    if (l->rows) l->rows[l->n] = row;
    if (l->cols) l->cols[l->n] = col;
    if (l->w) l->w[l->n] = w;
  }
  l->n++;
}

int64_t orc_jitconn_connections(int32_t kind, float p0, float p1, int32_t clen, uint32_t seed,
                                int64_t num_row, int64_t num_col, int32_t outdim_parallel,
                                int32_t variant, int64_t cap, int64_t* rows, int64_t* cols, float* w) {
  conn_list l = {0, cap, rows, cols, w};
  jitconn_walk(kind, p0, p1, clen, seed, num_row, num_col, outdim_parallel, variant, NULL,
               conn_list_visit, &l);
  return l.n;
}

typedef struct {
  int32_t vec_kind, outdim_parallel, variant, kind;
  float p0;
  const void* vec;
  double *out64, *abs64;
} mv_ctx;

/* Contribution of one connection (row <- col) to y[row].
 * vec_kind 0, bool events: w when events[col] (all kernels).
 * vec_kind 1, float events:
 *   GPU pull  multiplies by the event value  (_event_mv_prob_homo_outdim_parallel_gpu, :280)
 *   GPU push  adds w when events[col] != 0   (_event_mv_prob_homo_gpu, :242-250)
 *   CPU both  add w when events[col] != 0    (:182-188, :210-211)
 * vec_kind 2, dense vector (mv_prob_*): w * vector[col] (_matvec_taichi.py:73-76, :97-104, :133-137). */
static void mv_visit(void* ctx, int64_t row, int64_t col, float w) {
  mv_ctx* c = (mv_ctx*)ctx;
  double f;
  if (c->vec_kind == 0) {
    f = ((const uint8_t*)c->vec)[col] ? 1.0 : 0.0;
  } else if (c->vec_kind == 1) {
    float e = ((const float*)c->vec)[col];
    if (c->variant == 0 && c->outdim_parallel) f = (double)e;
    else f = (e != 0.0f) ? 1.0 : 0.0;
  } else {
    f = (double)((const float*)c->vec)[col];
  }
  double t = (double)w * f;
  c->out64[row] += t;
  if (c->abs64) {
    /* normal weights are mu + sigma*z: the rounding of that sum scales with |mu| + |sigma*z|,
       not with the (possibly cancelled) |w| */
    double scale = c->kind == 2 ? (fabs((double)c->p0) + fabs((double)w - (double)c->p0)) : fabs((double)w);
    c->abs64[row] += scale * fabs(f);
  }
}

void orc_jitconn_mv(int32_t kind, int32_t vec_kind, const void* vec, int64_t num_row, int64_t num_col,
                    float p0, float p1, int32_t clen, uint32_t seed, int32_t outdim_parallel,
                    int32_t variant, double* out64, double* abs64) {
  memset(out64, 0, sizeof(double) * (size_t)num_row);
  if (abs64) memset(abs64, 0, sizeof(double) * (size_t)num_row);
  uint8_t* active = NULL;
  if (!outdim_parallel && vec_kind != 2) {
    /* push kernels test the event before touching the stream */
    active = (uint8_t*)malloc((size_t)num_col);
    for (int64_t j = 0; j < num_col; ++j) {
      if (vec_kind == 0) active[j] = ((const uint8_t*)vec)[j] != 0;
      else active[j] = ((const float*)vec)[j] != 0.0f;
    }
  }
  mv_ctx c = {vec_kind, outdim_parallel, variant, kind, p0, vec, out64, abs64};
  jitconn_walk(kind, p0, p1, clen, seed, num_row, num_col, outdim_parallel, variant, active, mv_visit, &c);
  free(active);
}

/* orc_jitconn_mv with outdim_parallel = 1, restricted to the output rows flagged in row_mask:
 * in the pull form every output row draws its connections from its own stream (seeded by the
 * row), so a row's value does not depend on the others.  Unflagged rows are left at zero. */
void orc_jitconn_mv_rows(int32_t kind, int32_t vec_kind, const void* vec, int64_t num_row, int64_t num_col,
                         float p0, float p1, int32_t clen, uint32_t seed, int32_t variant,
                         const uint8_t* row_mask, double* out64, double* abs64) {
  memset(out64, 0, sizeof(double) * (size_t)num_row);
  if (abs64) memset(abs64, 0, sizeof(double) * (size_t)num_row);
  mv_ctx c = {vec_kind, 1, variant, kind, p0, vec, out64, abs64};
  jitconn_walk(kind, p0, p1, clen, seed, num_row, num_col, 1, variant, row_mask, mv_visit, &c);
}

/* ------------------------------------------------------------------------ */
/* event CSR and sparse CSR                                                  */
/* ------------------------------------------------------------------------ */

static inline int64_t ld_idx(const void* p, int32_t idx64, int64_t i) {
  return idx64 ? ((const int64_t*)p)[i] : (int64_t)((const int32_t*)p)[i];
}

static inline int ev_on(const void* events, int32_t ev_kind, int64_t i) {
  if (ev_kind == 0) return ((const uint8_t*)events)[i] != 0;
  float e = ((const float*)events)[i];
  return ev_kind == 1 ? (e > 0.0f) : (e != 0.0f);
}

/* brainpy/_src/math/event/_csr_matvec.py:321-412 (Numba CPU kernels):
 *   transpose:  for each active row i (row order), for j in row: out[indices[j]] += w_j
 *   otherwise:  out[i] = sum over j in row i with events[indices[j]] of w_j
 * The event value itself is never multiplied in (only its truth value is used). */
void orc_event_csrmv(const float* data, int64_t ndata, const void* indices, const void* indptr,
                     int32_t idx64, const void* events, int32_t ev_kind, int64_t m, int64_t n,
                     int32_t transpose, double* out64, double* abs64, float* out32, float* count32) {
  int64_t n_out = transpose ? n : m;
  int homo = ndata == 1;
  memset(out64, 0, sizeof(double) * (size_t)n_out);
  if (abs64) memset(abs64, 0, sizeof(double) * (size_t)n_out);
  if (out32) memset(out32, 0, sizeof(float) * (size_t)n_out);
  int64_t* cnt = NULL;
  if (count32 && homo) cnt = (int64_t*)calloc((size_t)n_out, sizeof(int64_t));
  for (int64_t i = 0; i < m; ++i) {
    int64_t b = ld_idx(indptr, idx64, i), e = ld_idx(indptr, idx64, i + 1);
    if (transpose) {
      if (!ev_on(events, ev_kind, i)) continue;
      for (int64_t j = b; j < e; ++j) {
        int64_t col = ld_idx(indices, idx64, j);
        float w = homo ? data[0] : data[j];
        out64[col] += (double)w;
        if (abs64) abs64[col] += fabs((double)w);
        if (out32) out32[col] += w;
        if (cnt) cnt[col] += 1;
      }
    } else {
      float r = 0.0f;
      for (int64_t j = b; j < e; ++j) {
        int64_t col = ld_idx(indices, idx64, j);
        if (!ev_on(events, ev_kind, col)) continue;
        float w = homo ? data[0] : data[j];
        out64[i] += (double)w;
        if (abs64) abs64[i] += fabs((double)w);
        r += w;
        if (cnt) cnt[i] += 1;
      }
      if (out32) out32[i] = r;
    }
  }
  if (cnt) {
    for (int64_t k = 0; k < n_out; ++k) count32[k] = (float)cnt[k] * data[0];
    free(cnt);
  }
}

/* brainpy/_src/math/sparse/_csr_mv.py:126-164 (Numba CPU kernels):
 *   transpose: out[indices[j]] += w_j * v[i];  otherwise out[i] = sum_j w_j * v[indices[j]] */
void orc_csrmv(const float* data, int64_t ndata, const void* indices, const void* indptr,
               int32_t idx64, const float* vec, int64_t m, int64_t n, int32_t transpose,
               double* out64, double* abs64, float* out32) {
  int64_t n_out = transpose ? n : m;
  int homo = ndata == 1;
  memset(out64, 0, sizeof(double) * (size_t)n_out);
  if (abs64) memset(abs64, 0, sizeof(double) * (size_t)n_out);
  if (out32) memset(out32, 0, sizeof(float) * (size_t)n_out);
  for (int64_t i = 0; i < m; ++i) {
    int64_t b = ld_idx(indptr, idx64, i), e = ld_idx(indptr, idx64, i + 1);
    if (transpose) {
      float v = vec[i];
      for (int64_t j = b; j < e; ++j) {
        int64_t col = ld_idx(indices, idx64, j);
        float w = homo ? data[0] : data[j];
        double t = (double)w * (double)v;
        out64[col] += t;
        if (abs64) abs64[col] += fabs(t);
        if (out32) out32[col] += w * v;
      }
    } else {
      float r = 0.0f;
      for (int64_t j = b; j < e; ++j) {
        int64_t col = ld_idx(indices, idx64, j);
        float w = homo ? data[0] : data[j];
        double t = (double)w * (double)vec[col];
        out64[i] += t;
        if (abs64) abs64[i] += fabs(t);
        r += w * vec[col];
      }
      if (out32) out32[i] = r;
    }
  }
}

/* brainpy/_src/math/event/_info_collection.py:144-155: ascending active indices, padded -1 */
int64_t orc_event_info(const uint8_t* events, int64_t n, int32_t* ids) {
  int64_t num = 0;
  for (int64_t i = 0; i < n; ++i) ids[i] = -1;
  for (int64_t i = 0; i < n; ++i)
    if (events[i]) ids[num++] = (int32_t)i;
  return num;
}

/* ------------------------------------------------------------------------ */
/* Plasticity on CSR / CSC (brainpy/_src/dnn/linear.py:650-698)              */
/* ------------------------------------------------------------------------ */

/* np.minimum(np.maximum(x, lo), hi): NaN stays NaN. */
static float clip_np(float x, float lo, float hi) {
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}

/* _cpu_csr_on_pre_update (linear.py:650-660): out = w; for every pre row i with spike[i],
 * out[k] = clip(out[k] + trace[indices[k]]) over the row's synapses k. */
void orc_csr_on_pre_update(const float* w, const void* indices, const void* indptr, int32_t idx64,
                           int64_t m, const uint8_t* spike, const float* trace, float w_min, float w_max,
                           int64_t nnz, float* out) {
  memcpy(out, w, sizeof(float) * (size_t)nnz);
  for (int64_t i = 0; i < m; ++i) {
    if (!spike[i]) continue;
    int64_t b = ld_idx(indptr, idx64, i), e = ld_idx(indptr, idx64, i + 1);
    for (int64_t k = b; k < e; ++k) out[k] = clip_np(out[k] + trace[ld_idx(indices, idx64, k)], w_min, w_max);
  }
}

/* _cpu_csc_on_pre_update (linear.py:675-686): out = w; for every post column i with spike[i],
 * out[w_ids[k]] = clip(out[w_ids[k]] + trace[pre_ids[k]]) over the column's entries k. */
void orc_csc_on_post_update(const float* w, const void* pre_ids, const void* indptr, const void* w_ids,
                            int32_t idx64, int64_t n, const uint8_t* spike, const float* trace, float w_min,
                            float w_max, int64_t nnz, float* out) {
  memcpy(out, w, sizeof(float) * (size_t)nnz);
  for (int64_t i = 0; i < n; ++i) {
    if (!spike[i]) continue;
    int64_t b = ld_idx(indptr, idx64, i), e = ld_idx(indptr, idx64, i + 1);
    for (int64_t k = b; k < e; ++k) {
      int64_t l = ld_idx(w_ids, idx64, k);
      out[l] = clip_np(out[l] + trace[ld_idx(pre_ids, idx64, k)], w_min, w_max);
    }
  }
}

/* csr2csc (brainpy/_src/connect/base.py:645-726) with data = arange(nnz): entries sorted by
 * column, stably (row order kept within a column).  Counting sort; outputs int64. */
void orc_csr2csc(const void* indices, const void* indptr, int32_t idx64, int64_t m, int64_t n,
                 int64_t* pre_ids, int64_t* c_indptr, int64_t* w_ids) {
  memset(c_indptr, 0, sizeof(int64_t) * (size_t)(n + 1));
  int64_t nnz = ld_idx(indptr, idx64, m);
  for (int64_t k = 0; k < nnz; ++k) c_indptr[ld_idx(indices, idx64, k) + 1]++;
  for (int64_t c = 0; c < n; ++c) c_indptr[c + 1] += c_indptr[c];
  int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  memcpy(cur, c_indptr, sizeof(int64_t) * (size_t)n);
  for (int64_t i = 0; i < m; ++i) {
    int64_t b = ld_idx(indptr, idx64, i), e = ld_idx(indptr, idx64, i + 1);
    for (int64_t k = b; k < e; ++k) {
      int64_t c = ld_idx(indices, idx64, k);
      int64_t p = cur[c]++;
      pre_ids[p] = i;
      w_ids[p] = k;
    }
  }
  free(cur);
}

/* ------------------------------------------------------------------------ */
/* FixedProb rows (the device generator's algorithm, serially)               */
/* ------------------------------------------------------------------------ */

static uint64_t orc_mix64(uint64_t x) { /* SplitMix64 finaliser (Steele et al. 2014) */
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return x;
}

/* Row `row` of FixedProb (brainpy/_src/connect/random_conn.py:73-128 for the law): the first K
 * distinct values (all K values with multi) of u(t) = mulhi(mix64(key + row*C1 + t*C2), n),
 * key = (seed + 1) * golden ratio; diagonal entries removed when drop_self.  Writes the kept
 * values in order and returns their number. */
int64_t orc_fixed_prob_row(uint64_t seed, int64_t row, int64_t n, int32_t K, int32_t multi, int32_t drop_self,
                           int32_t* out) {
  const uint64_t key = (seed + 1ull) * 0x9E3779B97F4A7C15ull;
  uint8_t* seen = multi ? NULL : (uint8_t*)calloc((size_t)(n > 0 ? n : 1), 1);
  int64_t count = 0, kept = 0;
  for (uint64_t t = 0; count < K; ++t) {
    uint64_t h = orc_mix64(key + (uint64_t)row * 0xD1B54A32D192ED03ull + t * 0x8CB92BA72F3D8DD7ull);
    uint32_t v = (uint32_t)(((unsigned __int128)h * (uint64_t)n) >> 64);
    if (!multi) {
      if (seen[v]) continue;
      seen[v] = 1;
    }
    ++count;
    if (drop_self && (int64_t)v == row) continue;
    out[kept++] = (int32_t)v;
  }
  free(seen);
  return kept;
}

/* ------------------------------------------------------------------------ */
/* LIF / Expon / COBA                                                        */
/* ------------------------------------------------------------------------ */

static double exprel64(double x) {
  if (fabs(x) <= 1e-8) return 1.0 + x / 2.0 + x * x / 6.0;
  return expm1(x) / x;
}

/* One neuron, float32 in the reference's operation order.
 * Expon (abstract_models.py:121-134): g += dg (add_current), then
 *   g <- g + (dt * exprel(dt * lin)) * ((-g) / tau), lin = d(-g/tau)/dg = -(1/tau).
 * LifRefLTC (lif.py:461-500 with derivative lif.py:254-256 and COBA outputs.py:53-54):
 *   I = (inp + ge*(Ee - V)) + gi*(Ei - V);  f = ((-V + V_rest) + R*I) / tau
 *   lin = dF/dV = (-1 - R*(ge + gi)) / tau   (LTC; LifRef: -(1/tau), lif.py:550-556)
 *   V' = V + (dt * exprel(dt * lin)) * f    (exponential.py:357-362)
 *   refractory: (t - t_last) <= tau_ref -> V' = V;  spike = V' >= V_th;
 *   V' = spike ? V_reset : V';  t_last = spike ? t : t_last. */
static void lif_neuron_f32(const orc_lif_params* p, float* V, float* ge, float* gi, float* t_last,
                           uint8_t* spike, float dge, float dgi, float t, float dt) {
  float g_e = *ge + dge;
  float g_i = *gi + dgi;
  {
    float lin = -(1.0f / p->tau_e);
    float phi = bp_exprel(dt * lin);
    float dtphi = dt * phi;
    g_e = g_e + dtphi * ((-g_e) / p->tau_e);
  }
  {
    float lin = -(1.0f / p->tau_i);
    float phi = bp_exprel(dt * lin);
    float dtphi = dt * phi;
    g_i = g_i + dtphi * ((-g_i) / p->tau_i);
  }
  float v = *V;
  float I = (p->input + g_e * (p->E_e - v)) + g_i * (p->E_i - v);
  float f = ((-v + p->V_rest) + p->R * I) / p->tau;
  float lin;
  if (p->ltc) lin = (-1.0f - p->R * (g_e + g_i)) / p->tau;
  else lin = -(1.0f / p->tau);
  float phi = bp_exprel(dt * lin);
  float vn = v + (dt * phi) * f;
  if ((t - *t_last) <= p->tau_ref) vn = v;
  uint8_t s = vn >= p->V_th;
  if (s) {
    vn = p->V_reset;
    *t_last = t;
  }
  *V = vn;
  *ge = g_e;
  *gi = g_i;
  *spike = s;
}

/* float64 arithmetic for the state update; time and the refractory test stay in float32
 * exactly as the reference computes them (t = f32(i) * f32(dt)), since they are discrete
 * bookkeeping rather than integration. */
static void lif_neuron_f64(const orc_lif_params* p, float* V, float* ge, float* gi, float* t_last,
                           uint8_t* spike, float dge, float dgi, float t, double dt) {
  double g_e = (double)*ge + (double)dge;
  double g_i = (double)*gi + (double)dgi;
  g_e = g_e + dt * exprel64(-dt / p->tau_e) * (-g_e / p->tau_e);
  g_i = g_i + dt * exprel64(-dt / p->tau_i) * (-g_i / p->tau_i);
  double v = *V;
  double I = p->input + g_e * (p->E_e - v) + g_i * (p->E_i - v);
  double f = (-v + p->V_rest + p->R * I) / p->tau;
  double lin = p->ltc ? (-1.0 - p->R * (g_e + g_i)) / p->tau : -1.0 / p->tau;
  double vn = v + dt * exprel64(dt * lin) * f;
  if ((t - *t_last) <= p->tau_ref) vn = v;
  uint8_t s = vn >= (double)p->V_th;
  if (s) {
    vn = p->V_reset;
    *t_last = t;
  }
  *V = (float)vn;
  *ge = (float)g_e;
  *gi = (float)g_i;
  *spike = s;
}

void orc_lif_step(const orc_lif_params* p, int64_t n, float* V, float* ge, float* gi,
                  float* t_last, uint8_t* spike, const float* dge, const float* dgi,
                  int32_t step_i, float dt, int32_t precise) {
  /* runners.py:624: t = t0 + i * dt with i int32 and dt float -> float32(i) * float32(dt) */
  float t = (float)step_i * dt;
  for (int64_t k = 0; k < n; ++k) {
    float a = dge ? dge[k] : 0.0f, b = dgi ? dgi[k] : 0.0f;
    if (precise) lif_neuron_f64(p, V + k, ge + k, gi + k, t_last + k, spike + k, a, b, t, (double)dt);
    else lif_neuron_f32(p, V + k, ge + k, gi + k, t_last + k, spike + k, a, b, t, dt);
  }
}

void orc_coba_net_run(const orc_lif_params* p, int64_t n, int64_t n_exc,
                      const int32_t* exc_indptr, const int32_t* exc_indices, float we,
                      const int32_t* inh_indptr, const int32_t* inh_indices, float wi,
                      float* V, float* ge, float* gi, float* t_last, uint8_t* spike,
                      int32_t step0, int32_t steps, float dt, int32_t count_mode,
                      int64_t* spike_counts, int32_t trace_steps, float* v_trace) {
  float* dge = (float*)calloc((size_t)n, sizeof(float));
  float* dgi = (float*)calloc((size_t)n, sizeof(float));
  int32_t* ce = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  int32_t* ci = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  for (int32_t s = 0; s < steps; ++s) {
    /* align_post.py:271-275: spikes of the previous step -> event.csrmv -> g += current */
    memset(dge, 0, sizeof(float) * (size_t)n);
    memset(dgi, 0, sizeof(float) * (size_t)n);
    memset(ce, 0, sizeof(int32_t) * (size_t)n);
    memset(ci, 0, sizeof(int32_t) * (size_t)n);
    for (int64_t r = 0; r < n_exc; ++r) {
      if (!spike[r]) continue;
      for (int32_t j = exc_indptr[r]; j < exc_indptr[r + 1]; ++j) {
        ce[exc_indices[j]] += 1;
        dge[exc_indices[j]] += we;
      }
    }
    for (int64_t r = 0; r < n - n_exc; ++r) {
      if (!spike[n_exc + r]) continue;
      for (int32_t j = inh_indptr[r]; j < inh_indptr[r + 1]; ++j) {
        ci[inh_indices[j]] += 1;
        dgi[inh_indices[j]] += wi;
      }
    }
    if (count_mode) {
      for (int64_t k = 0; k < n; ++k) {
        dge[k] = (float)ce[k] * we;
        dgi[k] = (float)ci[k] * wi;
      }
    }
    orc_lif_step(p, n, V, ge, gi, t_last, spike, dge, dgi, step0 + s, dt, 0);
    if (spike_counts) {
      int64_t c = 0;
      for (int64_t k = 0; k < n; ++k) c += spike[k];
      spike_counts[s] = c;
    }
    if (v_trace && s < trace_steps) memcpy(v_trace + (size_t)s * (size_t)n, V, sizeof(float) * (size_t)n);
  }
  free(dge);
  free(dgi);
  free(ce);
  free(ci);
}

/* The same network with synaptic delays on the pre-synaptic groups: VarDelay in its rotating
 * form (brainpy/_src/delay.py:334-373).  A projection with delay_step d = ceil(delay / dt)
 * reads, at step i, target.value when d == 0 and data[(d - i - 1) mod L] otherwise; after the
 * neurons update, the delay stores the new spikes at data[(-i - 1) mod L] (L = the longest
 * registered delay step; data starts at zero).  d_e applies to the excitatory rows, d_i to the
 * inhibitory rows; ring is data, L x n bytes, carried across calls; i = step0 + s. */
static int64_t pos_mod(int64_t a, int64_t L) { return ((a % L) + L) % L; }

void orc_coba_net_run_delayed(const orc_lif_params* p, int64_t n, int64_t n_exc,
                              const int32_t* exc_indptr, const int32_t* exc_indices, float we,
                              const int32_t* inh_indptr, const int32_t* inh_indices, float wi,
                              float* V, float* ge, float* gi, float* t_last, uint8_t* spike,
                              int32_t step0, int32_t steps, float dt, int32_t d_e, int32_t d_i,
                              int32_t L, uint8_t* ring, int64_t* spike_counts) {
  float* dge = (float*)calloc((size_t)n, sizeof(float));
  float* dgi = (float*)calloc((size_t)n, sizeof(float));
  int32_t* ce = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  int32_t* ci = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  for (int32_t s = 0; s < steps; ++s) {
    const int64_t i = (int64_t)step0 + s;
    const uint8_t* src_e = d_e == 0 ? spike : ring + pos_mod((int64_t)d_e - i - 1, L) * n;
    const uint8_t* src_i = d_i == 0 ? spike : ring + pos_mod((int64_t)d_i - i - 1, L) * n;
    memset(ce, 0, sizeof(int32_t) * (size_t)n);
    memset(ci, 0, sizeof(int32_t) * (size_t)n);
    for (int64_t r = 0; r < n_exc; ++r) {
      if (!src_e[r]) continue;
      for (int32_t j = exc_indptr[r]; j < exc_indptr[r + 1]; ++j) ce[exc_indices[j]] += 1;
    }
    for (int64_t r = 0; r < n - n_exc; ++r) {
      if (!src_i[n_exc + r]) continue;
      for (int32_t j = inh_indptr[r]; j < inh_indptr[r + 1]; ++j) ci[inh_indices[j]] += 1;
    }
    for (int64_t k = 0; k < n; ++k) {
      dge[k] = (float)ce[k] * we;
      dgi[k] = (float)ci[k] * wi;
    }
    orc_lif_step(p, n, V, ge, gi, t_last, spike, dge, dgi, (int32_t)i, dt, 0);
    if (L > 0) memcpy(ring + pos_mod(-i - 1, L) * n, spike, (size_t)n);
    if (spike_counts) {
      int64_t c = 0;
      for (int64_t k = 0; k < n; ++k) c += spike[k];
      spike_counts[s] = c;
    }
  }
  free(dge);
  free(dgi);
  free(ce);
  free(ci);
}

/* the shared deterministic exp / exprel (brainpy_gb300/csrc/bp_math.h), exported for tests */
float orc_bp_expf(float x) { return bp_expf(x); }
float orc_bp_exprel(float x) { return bp_exprel(x); }
