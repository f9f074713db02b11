"""ctypes wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY.  This package restates the reference's algorithms on
the CPU; it is imported by tests/, by __graft_entry__.smoke() and by the CPU
baseline leg of bench.py, to compare against.  The brainpy_gb300 package never
imports it.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_L = None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_U32 = ctypes.c_uint32
_F32 = ctypes.c_float


class LifParams(ctypes.Structure):
  _fields_ = [("V_rest", _F32), ("V_th", _F32), ("V_reset", _F32), ("tau", _F32), ("tau_ref", _F32),
              ("R", _F32), ("tau_e", _F32), ("tau_i", _F32), ("E_e", _F32), ("E_i", _F32),
              ("input", _F32), ("ltc", _I32)]


def build(force=False):
  """Compiles liboracle.so with the Makefile next to this file."""
  args = ["make", "-s", "-C", HERE]
  if force:
    subprocess.run(["make", "-s", "-C", HERE, "clean"], check=True)
  subprocess.run(args, check=True)
  return LIB_PATH


def lib():
  global _L
  if _L is None:
    if not os.path.exists(LIB_PATH):
      build()
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "orc_lfsr88_key": (None, [_U32, _P]),
        "orc_lfsr88_next_key": (None, [_P]),
        "orc_lfsr88_random_integers": (_I32, [_P, _I32, _I32]),
        "orc_lfsr88_uniform": (_F32, [_P, _F32, _F32]),
        "orc_lfsr88_normal": (_F32, [_P, _F32, _F32]),
        "orc_lfsr88_stream": (None, [_U32, _I32, _P]),
        "orc_jitconn_connections": (_I64, [_I32, _F32, _F32, _I32, _U32, _I64, _I64, _I32, _I32, _I64, _P, _P, _P]),
        "orc_jitconn_mv": (None, [_I32, _I32, _P, _I64, _I64, _F32, _F32, _I32, _U32, _I32, _I32, _P, _P]),
        "orc_jitconn_mv_rows": (None, [_I32, _I32, _P, _I64, _I64, _F32, _F32, _I32, _U32, _I32, _P, _P, _P]),
        "orc_event_csrmv": (None, [_P, _I64, _P, _P, _I32, _P, _I32, _I64, _I64, _I32, _P, _P, _P, _P]),
        "orc_csrmv": (None, [_P, _I64, _P, _P, _I32, _P, _I64, _I64, _I32, _P, _P, _P]),
        "orc_event_info": (_I64, [_P, _I64, _P]),
        "orc_csr_on_pre_update": (None, [_P, _P, _P, _I32, _I64, _P, _P, _F32, _F32, _I64, _P]),
        "orc_csc_on_post_update": (None, [_P, _P, _P, _P, _I32, _I64, _P, _P, _F32, _F32, _I64, _P]),
        "orc_csr2csc": (None, [_P, _P, _I32, _I64, _I64, _P, _P, _P]),
        "orc_fixed_prob_row": (_I64, [ctypes.c_uint64, _I64, _I64, _I32, _I32, _I32, _P]),
        "orc_lif_step": (None, [_P, _I64, _P, _P, _P, _P, _P, _P, _P, _I32, _F32, _I32]),
        "orc_coba_net_run": (None, [_P, _I64, _I64, _P, _P, _F32, _P, _P, _F32, _P, _P, _P, _P, _P, _I32, _I32,
                                    _F32, _I32, _P, _I32, _P]),
        "orc_coba_net_run_delayed": (None, [_P, _I64, _I64, _P, _P, _F32, _P, _P, _F32, _P, _P, _P, _P, _P, _I32,
                                            _I32, _F32, _I32, _I32, _I32, _P, _P]),
        "cpu_event_csrmv_bool": (None, [_P, _I64, _P, _P, _P, _I64, _I64, _I32, _P]),
        "cpu_event_csrmv_bool_t_batch": (_I32, [_P, _I64, _P, _P, _P, _I64, _I64, _I64, _P]),
        "cpu_num_threads": (_I32, []),
        "orc_bp_expf": (_F32, [_F32]),
        "orc_bp_exprel": (_F32, [_F32]),
    }
    for name, (res, args) in sig.items():
      f = getattr(L, name)
      f.restype = res
      f.argtypes = args
    _L = L
  return _L


def _p(a):
  return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


# ---- LFSR88 ------------------------------------------------------------------
def lfsr88_stream(seed, n):
  out = np.zeros(n, np.uint32)
  lib().orc_lfsr88_stream(seed, n, _p(out))
  return out


def lfsr88_sequence(seed, n, fn, *args):
  key = np.zeros(4, np.uint32)
  lib().orc_lfsr88_key(seed, _p(key))
  f = getattr(lib(), "orc_lfsr88_" + fn)
  return [f(_p(key), *args) for _ in range(n)]


# ---- jitconn -----------------------------------------------------------------
KINDS = {"homo": 0, "uniform": 1, "normal": 2}


def jitconn_connections(kind, p0, p1, clen, seed, num_row, num_col, outdim_parallel, variant="gpu"):
  v = 0 if variant == "gpu" else 1
  k = KINDS[kind]
  n = lib().orc_jitconn_connections(k, p0, p1, clen, seed, num_row, num_col, int(outdim_parallel), v, 0,
                                    None, None, None)
  rows = np.zeros(n, np.int64)
  cols = np.zeros(n, np.int64)
  w = np.zeros(n, np.float32)
  lib().orc_jitconn_connections(k, p0, p1, clen, seed, num_row, num_col, int(outdim_parallel), v, n,
                                _p(rows), _p(cols), _p(w))
  return rows, cols, w


def jitconn_mv(kind, vec, num_row, p0, p1, clen, seed, outdim_parallel, variant="gpu", vec_kind=None):
  """FP64 y = M v; returns (y64, abs64).  vec_kind: 0 bool events, 1 float events, 2 dense."""
  vec = np.ascontiguousarray(vec)
  if vec_kind is None:
    vec_kind = 0 if vec.dtype == np.bool_ else 2
  if vec.dtype == np.bool_:
    vec = vec.view(np.uint8)
  else:
    vec = vec.astype(np.float32, copy=False)
  out = np.zeros(num_row, np.float64)
  ab = np.zeros(num_row, np.float64)
  lib().orc_jitconn_mv(KINDS[kind], vec_kind, _p(vec), num_row, vec.shape[0], p0, p1, clen, seed,
                       int(outdim_parallel), 0 if variant == "gpu" else 1, _p(out), _p(ab))
  return out, ab


def jitconn_mv_rows(kind, vec, num_row, p0, p1, clen, seed, rows, variant="gpu", vec_kind=None):
  """Pull form (outdim_parallel) of jitconn_mv for the output rows `rows` only: returns
  (y64[rows], abs64[rows])."""
  vec = np.ascontiguousarray(vec)
  if vec_kind is None:
    vec_kind = 0 if vec.dtype == np.bool_ else 2
  vec = vec.view(np.uint8) if vec.dtype == np.bool_ else vec.astype(np.float32, copy=False)
  mask = np.zeros(num_row, np.uint8)
  mask[np.asarray(rows)] = 1
  out = np.zeros(num_row, np.float64)
  ab = np.zeros(num_row, np.float64)
  lib().orc_jitconn_mv_rows(KINDS[kind], vec_kind, _p(vec), num_row, vec.shape[0], p0, p1, clen, seed,
                            0 if variant == "gpu" else 1, _p(mask), _p(out), _p(ab))
  return out[rows], ab[rows]


# ---- CSR ---------------------------------------------------------------------
EV_BOOL, EV_F32_POS, EV_F32_NZ = 0, 1, 2


def event_csrmv(data, indices, indptr, events, shape, transpose, ev_rule=EV_F32_POS):
  """Returns dict(out64, abs64, out32 (reference loop order), count32 (homo only))."""
  data = np.ascontiguousarray(np.atleast_1d(data).astype(np.float32))
  idx64 = 1 if indices.dtype == np.int64 else 0
  it = np.int64 if idx64 else np.int32
  indices = np.ascontiguousarray(indices.astype(it))
  indptr = np.ascontiguousarray(indptr.astype(it))
  events = np.ascontiguousarray(events)
  if events.dtype == np.bool_:
    ek, ev = EV_BOOL, events.view(np.uint8)
  else:
    ek, ev = ev_rule, events.astype(np.float32)
  m, n = shape
  n_out = n if transpose else m
  o64 = np.zeros(n_out, np.float64)
  a64 = np.zeros(n_out, np.float64)
  o32 = np.zeros(n_out, np.float32)
  c32 = np.zeros(n_out, np.float32) if data.shape[0] == 1 else None
  lib().orc_event_csrmv(_p(data), data.shape[0], _p(indices), _p(indptr), idx64, _p(ev), ek, m, n,
                        int(transpose), _p(o64), _p(a64), _p(o32), _p(c32))
  return {"out64": o64, "abs64": a64, "out32": o32, "count32": c32}


def csrmv(data, indices, indptr, vec, shape, transpose):
  data = np.ascontiguousarray(np.atleast_1d(data).astype(np.float32))
  idx64 = 1 if indices.dtype == np.int64 else 0
  it = np.int64 if idx64 else np.int32
  indices = np.ascontiguousarray(indices.astype(it))
  indptr = np.ascontiguousarray(indptr.astype(it))
  vec = np.ascontiguousarray(vec.astype(np.float32))
  m, n = shape
  n_out = n if transpose else m
  o64 = np.zeros(n_out, np.float64)
  a64 = np.zeros(n_out, np.float64)
  o32 = np.zeros(n_out, np.float32)
  lib().orc_csrmv(_p(data), data.shape[0], _p(indices), _p(indptr), idx64, _p(vec), m, n, int(transpose),
                  _p(o64), _p(a64), _p(o32))
  return {"out64": o64, "abs64": a64, "out32": o32}


def _idx(a):
  it = np.int64 if a.dtype == np.int64 else np.int32
  return np.ascontiguousarray(a.astype(it)), 1 if it == np.int64 else 0


def csr_on_pre_update(w, indices, indptr, spike, trace, w_min=-np.inf, w_max=np.inf):
  """brainpy/_src/dnn/linear.py:650-671 (numba loop): a new weight array."""
  w = np.ascontiguousarray(w, np.float32)
  ind, i64 = _idx(indices)
  ptr, _ = _idx(indptr.astype(ind.dtype))
  sp = np.ascontiguousarray(np.asarray(spike) != 0).view(np.uint8)
  tr = np.ascontiguousarray(trace, np.float32)
  out = np.empty_like(w)
  lib().orc_csr_on_pre_update(_p(w), _p(ind), _p(ptr), i64, ptr.shape[0] - 1, _p(sp), _p(tr), w_min, w_max,
                              w.shape[0], _p(out))
  return out


def csc_on_post_update(w, pre_ids, indptr, w_ids, spike, trace, w_min=-np.inf, w_max=np.inf):
  """brainpy/_src/dnn/linear.py:675-696 (numba loop): a new weight array."""
  w = np.ascontiguousarray(w, np.float32)
  pid, i64 = _idx(pre_ids)
  it = pid.dtype
  ptr = np.ascontiguousarray(indptr.astype(it))
  wid = np.ascontiguousarray(w_ids.astype(it))
  sp = np.ascontiguousarray(np.asarray(spike) != 0).view(np.uint8)
  tr = np.ascontiguousarray(trace, np.float32)
  out = np.empty_like(w)
  lib().orc_csc_on_post_update(_p(w), _p(pid), _p(ptr), _p(wid), i64, ptr.shape[0] - 1, _p(sp), _p(tr), w_min,
                               w_max, w.shape[0], _p(out))
  return out


def csr2csc(indices, indptr, n):
  """(pre_ids, indptr, w_ids) of brainpy/_src/connect/base.py:645-726 with data = arange(nnz)."""
  ind, i64 = _idx(indices)
  ptr = np.ascontiguousarray(indptr.astype(ind.dtype))
  m = ptr.shape[0] - 1
  nnz = int(ptr[-1]) if m >= 0 and ptr.size else 0
  pre = np.zeros(nnz, np.int64)
  cptr = np.zeros(n + 1, np.int64)
  wid = np.zeros(nnz, np.int64)
  lib().orc_csr2csc(_p(ind), _p(ptr), i64, m, n, _p(pre), _p(cptr), _p(wid))
  return pre, cptr, wid


def fixed_prob_rows(seed, rows, n, K, multi=False, drop_self=False):
  """The device FixedProb generator's rows, serially: list of int32 arrays."""
  out = []
  buf = np.zeros(max(K, 1), np.int32)
  for r in rows:
    k = lib().orc_fixed_prob_row(int(seed), int(r), int(n), int(K), int(multi), int(drop_self), _p(buf))
    out.append(buf[:k].copy())
  return out


def event_info(events):
  ev = np.ascontiguousarray(events.astype(np.bool_)).view(np.uint8)
  ids = np.zeros(ev.shape[0], np.int32)
  num = lib().orc_event_info(_p(ev), ev.shape[0], _p(ids))
  return ids, num


# ---- LIF / network -------------------------------------------------------------
def lif_params(V_rest=-60., V_th=-50., V_reset=-60., tau=20., tau_ref=5., R=1., tau_e=5., tau_i=10.,
               E_e=0., E_i=-80., input=20., ltc=True):
  return LifParams(V_rest, V_th, V_reset, tau, tau_ref, R, tau_e, tau_i, E_e, E_i, input, int(ltc))


def lif_step(params, V, ge, gi, t_last, spike, dge, dgi, step_i, dt, precise=False):
  """In-place on the numpy state arrays (float32 / uint8)."""
  lib().orc_lif_step(ctypes.byref(params), V.shape[0], _p(V), _p(ge), _p(gi), _p(t_last), _p(spike),
                     _p(dge), _p(dgi), step_i, dt, int(precise))


def coba_net_run(params, n, n_exc, exc_indptr, exc_indices, we, inh_indptr, inh_indices, wi, state, step0,
                 steps, dt, count_mode=True, trace_steps=0):
  """state: dict of numpy arrays V, ge, gi, t_last (float32), spike (uint8); updated in place.
  Returns (spike_counts per step, V trace)."""
  counts = np.zeros(steps, np.int64)
  trace = np.zeros((trace_steps, n), np.float32) if trace_steps else None
  lib().orc_coba_net_run(ctypes.byref(params), n, n_exc, _p(exc_indptr), _p(exc_indices), we, _p(inh_indptr),
                         _p(inh_indices), wi, _p(state["V"]), _p(state["ge"]), _p(state["gi"]),
                         _p(state["t_last"]), _p(state["spike"]), step0, steps, dt, int(count_mode),
                         _p(counts), trace_steps, _p(trace))
  return counts, trace


def delay_steps(delay, dt):
  """delay_step of brainpy/_src/delay.py:259-264: None -> 0, else ceil(delay / dt) in double."""
  return 0 if delay is None else int(math.ceil(float(delay) / float(dt)))


def coba_net_run_delayed(params, n, n_exc, exc_indptr, exc_indices, we, inh_indptr, inh_indices, wi, state, step0,
                         steps, dt, d_e, d_i):
  """The network with delay steps d_e / d_i on the excitatory / inhibitory rows (VarDelay,
  rotating).  state additionally carries "ring" (uint8 [L, n], L = max(d_e, d_i), created
  at zero when missing); updated in place.  Returns spike counts per step."""
  L = max(d_e, d_i)
  if L > 0 and state.get("ring") is None:
    state["ring"] = np.zeros((L, n), np.uint8)
  ring = state.get("ring") if L > 0 else None
  counts = np.zeros(steps, np.int64)
  lib().orc_coba_net_run_delayed(ctypes.byref(params), n, n_exc, _p(exc_indptr), _p(exc_indices), we,
                                 _p(inh_indptr), _p(inh_indices), wi, _p(state["V"]), _p(state["ge"]),
                                 _p(state["gi"]), _p(state["t_last"]), _p(state["spike"]), step0, steps, dt, d_e,
                                 d_i, L, _p(ring) if ring is not None else None, _p(counts))
  return counts


def cpu_event_csrmv_bool(data, indices, indptr, events, shape, transpose, out=None):
  """The restated reference CPU loop (the timed CPU baseline)."""
  data = np.ascontiguousarray(np.atleast_1d(data).astype(np.float32))
  m, n = shape
  if out is None:
    out = np.zeros(n if transpose else m, np.float32)
  lib().cpu_event_csrmv_bool(_p(data), data.shape[0], _p(indices), _p(indptr), _p(events.view(np.uint8)), m, n,
                             int(transpose), _p(out))
  return out


def cpu_event_csrmv_bool_t_batch(data, indices, indptr, events_batch, shape, out=None):
  """Independent transpose calls of the restated reference loop, one per host thread;
  returns (out (nb, n), threads used)."""
  data = np.ascontiguousarray(np.atleast_1d(data).astype(np.float32))
  m, n = shape
  ev = np.ascontiguousarray(events_batch).view(np.uint8)
  nb = ev.shape[0]
  if out is None:
    out = np.zeros((nb, n), np.float32)
  used = lib().cpu_event_csrmv_bool_t_batch(_p(data), data.shape[0], _p(indices), _p(indptr), _p(ev), nb, m, n,
                                            _p(out))
  return out, used


def cpu_num_threads():
  return lib().cpu_num_threads()
