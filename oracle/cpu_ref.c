/*
 * cpu_ref.c -- the reference's own CPU loops for event.csrmv, restated in C so
 * that they can be timed on the host cores as the CPU baseline (the reference's
 * Numba/JAX stack is not installable here).  TEST/BENCH INFRASTRUCTURE ONLY.
 *
 * Compiled with -O3 -ffast-math to mirror numba.njit(fastmath=True).  Threading
 * mirrors the reference: the transpose (scatter) kernel is a plain njit loop and
 * runs serially; the non-transpose kernel uses numba.prange over rows and runs
 * under OpenMP here.
 */
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle.h"

/* brainpy/_src/math/event/_csr_matvec.py:321-339 (transpose, bool events)
 * brainpy/_src/math/event/_csr_matvec.py:363-386 (non-transpose, bool events) */
void cpu_event_csrmv_bool(const float* data, int64_t ndata, const int32_t* indices,
                          const int32_t* indptr, const uint8_t* events, int64_t m, int64_t n,
                          int32_t transpose, float* out) {
  if (transpose) {
    memset(out, 0, sizeof(float) * (size_t)n);
    if (ndata > 1) {
      for (int64_t i = 0; i < m; ++i) {
        if (!events[i]) continue;
        for (int32_t j = indptr[i]; j < indptr[i + 1]; ++j) out[indices[j]] += data[j];
      }
    } else {
      const float w = data[0];
      for (int64_t i = 0; i < m; ++i) {
        if (!events[i]) continue;
        for (int32_t j = indptr[i]; j < indptr[i + 1]; ++j) out[indices[j]] += w;
      }
    }
  } else {
    if (ndata > 1) {
      /* the heterogeneous non-transpose loop is a plain range in the reference (:369-376) */
      for (int64_t i = 0; i < m; ++i) {
        float r = 0.0f;
        for (int32_t j = indptr[i]; j < indptr[i + 1]; ++j)
          if (events[indices[j]]) r += data[j];
        out[i] = r;
      }
    } else {
      const float w = data[0];
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < m; ++i) {
        float r = 0.0f;
        for (int32_t j = indptr[i]; j < indptr[i + 1]; ++j)
          if (events[indices[j]]) r += w;
        out[i] = r;
      }
    }
  }
}

/* Independent calls of the serial transpose loop (bool events), one per thread: the
 * reference's per-call path run concurrently on every host core, e.g. several simulations or
 * trials at once.  events: nb vectors of m; out: nb vectors of n.  Returns the threads used. */
int32_t cpu_event_csrmv_bool_t_batch(const float* data, int64_t ndata, const int32_t* indices,
                                     const int32_t* indptr, const uint8_t* events, int64_t nb, int64_t m,
                                     int64_t n, float* out) {
  int32_t used = 1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t b = 0; b < nb; ++b) {
#ifdef _OPENMP
    if (b == 0) used = (int32_t)omp_get_num_threads();
#endif
    cpu_event_csrmv_bool(data, ndata, indices, indptr, events + b * m, m, n, 1, out + b * n);
  }
  return used;
}

int32_t cpu_num_threads(void) {
#ifdef _OPENMP
  return (int32_t)omp_get_max_threads();
#else
  return 1;
#endif
}
