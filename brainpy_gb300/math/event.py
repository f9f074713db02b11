"""brainpy.math.event on GB300: csrmv, csrmv_taichi, info.

Signatures, argument checks and error types follow
brainpy/_src/math/event/_csr_matvec.py:38-110 (csrmv),
brainpy/_src/math/event/_csr_matvec_taichi.py:344-452 (csrmv_taichi) and
brainpy/_src/math/event/_info_collection.py:24-43 (info).
"""
import ctypes
import math
import os
import weakref
from typing import Optional, Tuple, Union

import torch

from .. import _lib
from .. import tuning
from . import _grad
from ._utils import as_tensor, default_device, event_type, float_data, index_type

__all__ = ["csrmv", "csrmv_taichi", "csrmv_batch", "info", "CSRPlan", "prepare", "autotune", "release_plans",
           "plan_cache_bytes"]


def fix_point_params(bound):
  """(k, tau) of a fixed-weight plan whose largest column sum of |w| is `bound`.  k is the
  largest exponent with bound * 2^k <= 2^31 - 2^24: a column's integer weights q = rint(w * 2^k)
  then add up below 2^31 in magnitude, the 2^24 covering the rounding of up to 2^25 entries a
  column (0 <= k <= 100; k = 30 for an all-zero matrix).  A weight with |w| >= tau =
  2^-(k+1) / 5e-6 is carried within 5e-6 of itself (|q * 2^-k - w| <= 2^-(k+1)); the nonzero
  weights below tau go to the plan's float side list."""
  k = 30 if bound <= 0.0 else int(math.floor(math.log2((2.0 ** 31 - 2.0 ** 24) / bound)))
  k = max(0, min(k, 100))
  return k, float(2.0 ** -(k + 1) / 5e-6)


def fix_fits_24(wmax, k):
  """Whether every integer weight rint(w * 2^k), |w| <= wmax, fits 24 bits (the 40-byte chunk
  records): wmax * 2^k < 2^23 - 1 keeps the rounded magnitude below 2^23."""
  return wmax * 2.0 ** k < 2.0 ** 23 - 1


class CSRPlan:
  """Column-tiled layout of a CSR matrix for the event-driven (transpose) kernels.

  Built once on the GPU from (indices, indptr[, heterogeneous data]); afterwards every
  ``csrmv(..., transpose=True)`` on the same matrix streams tile-local uint16 indices and
  accumulates in shared memory (see include/bpgpu.h, bp_csr_plan).  The plan holds its
  own device memory; it is a function of the arrays at build time.
  """

  def __init__(self, indices, indptr, shape, data=None, tile_w=None, cluster=4, kind="general", fix_record=None):
    dev = indices.device
    self.shape = (int(shape[0]), int(shape[1]))
    self.cluster = int(cluster)
    m, n = self.shape
    L = _lib.lib()
    heter = data is not None and data.numel() > 1
    if kind not in ("general", "count", "fixed"):
      raise ValueError(f"plan kind must be 'general', 'count' or 'fixed', got {kind!r}")
    if kind == "fixed" and not heter:
      raise ValueError("a fixed-weight plan needs per-synapse weights")
    if fix_record not in (None, 40, 48):
      raise ValueError(f"fix_record must be None, 40 or 48, got {fix_record!r}")
    # "count": tiles of up to 65,472 columns with 16-bit counters and per-tile partial counts
    # (event products with a homogeneous weight, one vector a call); "general": tiles whose
    # 32-bit accumulator fits one CTA (every product, batches, weights)
    if kind == "count" and tile_w is None and not heter:
      tile_w = L.bp_csr_plan_count_tile(n) or None
    if tile_w is None:
      if kind == "count":
        kind = "general"  # too few columns for a counting tile
      tile_w = L.bp_csr_plan_default_tile(n, self.cluster)
      if tile_w <= 0:
        raise _lib.BPError("bp_csr_plan_default_tile failed: " + L.bp_last_error().decode())
    self.kind = kind
    self.tile_w = int(tile_w)
    nbytes = L.bp_csr_plan_bytes(m, n, indices.numel(), int(heter), self.tile_w)
    self.mem = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
    self.c = _lib.CsrPlan()
    itype = index_type(indices, "indices")
    st = L.bp_csr_plan_build(_lib.ptr(data) if heter else None, data.numel() if heter else 1, _lib.ptr(indices),
                             _lib.ptr(indptr), itype, indices.numel(), m, n, self.tile_w, _lib.ptr(self.mem),
                             nbytes, ctypes.byref(self.c), _lib.stream_handle(dev))
    _lib.check(st, "csr_plan_build")
    if kind == "count":
      self.c.kind = 1
    self.heter = bool(heter)
    self.device = dev
    self.side = None
    if kind == "fixed":
      self._fix_weights(data, indices, n, fix_record if fix_record is not None else _FIX_RECORD)
    # per-call state kept ready: the C plan struct, a unit weight, and one workspace per stream
    # (calls on one stream are ordered, so they can share it)
    self._L = L
    self._cref = ctypes.byref(self.c)
    self._one = torch.ones(1, dtype=torch.float32, device=dev)
    self._ws_bytes = L.bp_event_csrmv_planned_workspace_size(self._cref)
    self._ws = {}

  def _fix_weights(self, data, indices, n, record=None):
    """Fixed-point weights: k from the largest column sum of |w| (no column's sum times 2^k
    reaches 2^31 - 2^24), tau = 2^-(k+1) / 5e-6; the weights below tau go to the side list,
    sorted by row.  The chunks are stored as 40-byte records (24-bit weights) when every
    max |w| * 2^k < 2^23 - 1 and `record` is not 48, else as 48-byte records (int32 weights);
    both give the same sums bit for bit."""
    L = _lib.lib()
    dev = self.device
    colsum = torch.zeros(max(n, 1), dtype=torch.float64, device=dev)
    colsum.index_add_(0, indices.to(torch.int64), data.abs().to(torch.float64))
    bound = float(colsum.max()) if colsum.numel() else 0.0
    k, tau = fix_point_params(bound)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    sp = _lib.stream_handle(dev)
    _lib.check(L.bp_csr_plan_fix_weights(ctypes.byref(self.c), k, tau, None, None, None, 0, _lib.ptr(cnt), 0, sp),
               "csr_plan_fix_weights")
    count = int(cnt.item())
    rows = torch.empty(max(count, 1), dtype=torch.int32, device=dev)
    cols = torch.empty(max(count, 1), dtype=torch.int32, device=dev)
    ws = torch.empty(max(count, 1), dtype=torch.float32, device=dev)
    _lib.check(L.bp_csr_plan_fix_weights(ctypes.byref(self.c), k, tau, _lib.ptr(rows), _lib.ptr(cols), _lib.ptr(ws),
                                         count, _lib.ptr(cnt), 1, sp), "csr_plan_fix_weights")
    order = torch.argsort(rows[:count].to(torch.int64), stable=True)
    rows, cols, ws = rows[:count][order], cols[:count][order], ws[:count][order]
    # the rows that hold side entries, each with its range of entries
    urows, per_row = torch.unique_consecutive(rows, return_counts=True)
    ptr = torch.zeros(urows.numel() + 1, dtype=torch.int32, device=dev)
    if count:
      ptr[1:] = torch.cumsum(per_row, 0).to(torch.int32)
    self.side = (urows.to(torch.int32).contiguous(), ptr, cols.contiguous(), ws.contiguous(), int(urows.numel()))
    self.side_entries = count
    self.fix_exponent, self.fix_tau = k, tau
    self.kind = "fixed"
    # the chunks as records (indices, integer weights): one read a segment
    wmax = float(data.abs().max()) if data.numel() else 0.0
    rec = 40 if record != 48 and fix_fits_24(wmax, k) else 48
    if record == 40 and rec != 40:
      raise ValueError(f"40-byte records need max |w| * 2^k < 2^23 - 1 (max |w| = {wmax}, k = {k})")
    fxb = int(L.bp_csr_plan_fix_interleave_bytes(ctypes.byref(self.c), rec))
    self.fx = torch.empty(max(fxb, 16), dtype=torch.uint8, device=dev)
    cnt.zero_()
    _lib.check(L.bp_csr_plan_fix_interleave(ctypes.byref(self.c), rec, _lib.ptr(self.fx), self.fx.numel(),
                                            _lib.ptr(cnt), sp), "csr_plan_fix_interleave")
    if rec == 40 and int(cnt.item()):
      raise _lib.BPError(f"csr_plan_fix_interleave: {int(cnt.item())} weights outside 24 bits")
    self.fix_record = rec

  def _workspace(self, stream_ptr, nbytes=None):
    nbytes = self._ws_bytes if nbytes is None else nbytes
    ws = self._ws.get(stream_ptr)
    if ws is None or ws.numel() < nbytes:
      ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=self.device)
      self._ws[stream_ptr] = ws
    return ws

  def csrmv(self, events, data=None, out=None, float_rule=_lib.BP_EV_F32_POS):
    """out (n) = event-driven transpose product on this plan."""
    etype, ev = event_type(events, float_rule)
    m, n = self.shape
    if ev.shape[0] != m:
      raise ValueError(f"Shape mismatch, vec ({ev.shape[0]},) @ mat {self.shape}.")
    if out is None:
      out = torch.empty(n, dtype=torch.float32, device=self.device)
    w = 0
    if not self.heter:
      w = (data if data is not None else self._one).data_ptr()
    sp = _lib.raw_stream(self.device)
    if self.side is not None:
      urows, ptr, cols, ws, nrows = self.side
      st = self._L.bp_event_csrmv_planned_fixed(self._cref, self.fx.data_ptr(), self.fix_record, urows.data_ptr(),
                                                ptr.data_ptr(), cols.data_ptr(), ws.data_ptr(), nrows, ev.data_ptr(),
                                                etype, out.data_ptr(), self.cluster, self._workspace(sp).data_ptr(),
                                                self._ws_bytes, sp)
      if st:
        _lib.check(st, "event_csrmv_planned_fixed")
      return out
    st = self._L.bp_event_csrmv_planned(self._cref, w, ev.data_ptr(), etype, out.data_ptr(), self.cluster,
                                        self._workspace(sp).data_ptr(), self._ws_bytes, sp)
    if st:
      _lib.check(st, "event_csrmv_planned")
    return out


  @staticmethod
  def variants():
    """Codes of the compiled tiled-kernel variants (G | RND << 8: lanes per segment, 16-byte
    chunks per lane and round)."""
    L = _lib.lib()
    k = L.bp_csr_plan_variants(None, 0)
    buf = (ctypes.c_int32 * k)()
    L.bp_csr_plan_variants(buf, k)
    return list(buf)

  @property
  def variant(self):
    """The kernel variant this plan runs (0: chosen from the mean segment length)."""
    return int(self.c.variant)

  @variant.setter
  def variant(self, code):
    self.c.variant = int(code)

  def autotune(self, events, data=None, candidates=None, reps=10):
    """Times every candidate variant (default: all compiled ones) on `events` -- a spike
    vector of the rate the model runs at -- and keeps the fastest for this plan.  Returns
    {variant code: microseconds per call}.  Every variant computes the same result."""
    m, n = self.shape
    out = torch.empty(n, dtype=torch.float32, device=self.device)
    times = {}
    for code in (candidates or self.variants()):
      self.c.variant = int(code)
      for _ in range(2):
        self.csrmv(events, data, out=out)
      t0 = torch.cuda.Event(enable_timing=True)
      t1 = torch.cuda.Event(enable_timing=True)
      t0.record()
      for _ in range(reps):
        self.csrmv(events, data, out=out)
      t1.record()
      t1.synchronize()
      times[int(code)] = t0.elapsed_time(t1) * 1e3 / reps
    self.c.variant = min(times, key=times.get)
    return times

  def csrmv_batch(self, events, data=None, out=None, float_rule=_lib.BP_EV_F32_POS):
    """out (B, n): row b is csrmv(events[b]); one launch pair for the whole batch."""
    return self._batch(events, data, out, float_rule, dense=False)

  def sparse_t_batch(self, vectors, data=None, out=None):
    """out (B, n): row b is sparse_t(vectors[b]); one launch pair for the whole batch."""
    return self._batch(vectors, data, out, _lib.BP_EV_F32_NZ, dense=True)

  def _batch(self, x, data, out, float_rule, dense):
    m, n = self.shape
    if x.ndim != 2 or x.shape[1] != m:
      raise ValueError(f"Shape mismatch, batch {tuple(x.shape)} @ mat {self.shape}.")
    x = x.contiguous()
    if dense:
      if x.dtype == torch.bool:
        x = x.to(torch.float32)
      if x.dtype != torch.float32:
        raise TypeError(f"vector must be float32, got {x.dtype}")
      etype, xv = _lib.BP_EV_F32_NZ, x
    else:
      etype, xv = event_type(x, float_rule)
    b = int(x.shape[0])
    if out is None:
      out = torch.empty((b, n), dtype=torch.float32, device=self.device)
    w = 0
    if not self.heter:
      w = (data if data is not None else self._one).data_ptr()
    sp = _lib.raw_stream(self.device)
    need = self._L.bp_event_csrmv_planned_batch_workspace_size(self._cref, b)
    ws = self._workspace(sp, need)
    if dense:
      st = self._L.bp_csrmv_planned_batch(self._cref, w, xv.data_ptr(), b, out.data_ptr(), self.cluster,
                                          ws.data_ptr(), ws.numel(), sp)
    else:
      st = self._L.bp_event_csrmv_planned_batch(self._cref, w, xv.data_ptr(), etype, b, out.data_ptr(),
                                                self.cluster, ws.data_ptr(), ws.numel(), sp)
    if st:
      _lib.check(st, "csrmv_planned_batch")
    return out

  def sparse_n(self, vector, data=None, out=None):
    """out (m) = A vector on this plan (sparse.csrmv, transpose=False): column tiles of the
    vector staged in shared memory, per-tile partial row sums added in tile order."""
    m, n = self.shape
    if vector.shape[0] != n:
      raise ValueError(f"Shape mismatch, mat {self.shape} @ vec ({vector.shape[0]},).")
    if out is None:
      out = torch.empty(m, dtype=torch.float32, device=self.device)
    w = 0
    if not self.heter:
      w = (data if data is not None else self._one).data_ptr()
    sp = _lib.raw_stream(self.device)
    need = self._L.bp_csrmv_planned_n_workspace_size(self._cref)
    key = ("n", sp)
    ws = self._ws.get(key)
    if ws is None or ws.numel() < need:
      ws = torch.empty(max(need, 1), dtype=torch.uint8, device=self.device)
      self._ws[key] = ws
    st = self._L.bp_csrmv_planned_n(self._cref, w, vector.data_ptr(), out.data_ptr(), ws.data_ptr(), ws.numel(), sp)
    if st:
      _lib.check(st, "csrmv_planned_n")
    return out

  def sparse_t(self, vector, data=None, out=None):
    """out (n) = A^T vector on this plan (sparse.csrmv, transpose=True)."""
    dev = self.device
    m, n = self.shape
    if vector.shape[0] != m:
      raise ValueError(f"Shape mismatch, vec ({vector.shape[0]},) @ mat {self.shape}.")
    if out is None:
      out = torch.empty(n, dtype=torch.float32, device=dev)
    w = 0
    if not self.heter:
      w = (data if data is not None else self._one).data_ptr()
    sp = _lib.raw_stream(dev)
    st = self._L.bp_csrmv_planned(self._cref, w, vector.data_ptr(), out.data_ptr(), self.cluster,
                                  self._workspace(sp).data_ptr(), self._ws_bytes, sp)
    if st:
      _lib.check(st, "csrmv_planned")
    return out


def prepare(indices, indptr, *, shape, data=None, tile_w=None, cluster=4) -> CSRPlan:
  """Builds the tiled plan of a CSR matrix (heterogeneous when `data` has nse entries)."""
  dev = indices.device if isinstance(indices, torch.Tensor) and indices.is_cuda else default_device()
  indices = as_tensor(indices, dev)
  indptr = as_tensor(indptr, dev)
  d = None
  if data is not None:
    d = float_data(data, dev)
  return CSRPlan(indices, indptr, shape, d, tile_w, cluster)


# ---- automatic plan cache ---------------------------------------------------------
# Keyed by the identity of the CSR tensors (and of heterogeneous weights) and the plan kind.
# Every entry remembers the tensors' version counters: an in-place change of any of them
# (STDP updates of the weights, for instance) replaces the entry, so the stale plan's memory
# is released at once instead of staying beside the new one.  _ROUTES holds, under the
# matrix key, the kernel family `autotune` chose ("row", "tiled" or "split"); a matrix without
# a route takes a plan from the size thresholds below.  `release_plans()` drops everything.
_PLANS = {}   # (matrix key, kind) -> (weak refs, versions, CSRPlan)
_ROUTES = {}  # matrix key -> (weak refs, versions, route)
_PLAN_MIN_N = int(os.environ.get("BPGPU_PLAN_MIN_N", 1 << 15))
_PLAN_MIN_NNZ = int(os.environ.get("BPGPU_PLAN_MIN_NNZ", 1 << 20))
_PLAN_DISABLE = os.environ.get("BPGPU_DISABLE_PLAN", "0") == "1"
# homogeneous event products on at least this many columns take the counting plan by default
# (BPGPU_SPLIT_MIN_N; off unless set: the autotuner times it against the general plan and
# routes a matrix to it when it wins)
_SPLIT_MIN_N = int(os.environ.get("BPGPU_SPLIT_MIN_N", 1 << 62))
# per-synapse weights take the fixed-point plan whenever the plan path is taken (N = 1e6,
# fan-out 1000, 2 %: 51.4 against 61.1 us a call); BPGPU_FIXED_MIN_N raises the threshold
_FIXED_MIN_N = int(os.environ.get("BPGPU_FIXED_MIN_N", 0))
# chunk records of fixed-weight plans: 0 picks 40 bytes (24-bit weights) where the weights fit,
# 48 (BPGPU_FIX_RECORD=48) keeps int32 weights
_FIX_RECORD = int(os.environ.get("BPGPU_FIX_RECORD", 0)) or None


def _ident(t):
  return (id(t), t.data_ptr())


def _matrix_key(data, indices, indptr, m, n):
  heter = data.numel() > 1
  return (_ident(indices), _ident(indptr), int(m), int(n), _ident(data) if heter else None)


def _versions(data, indices, indptr):
  return (indices._version, indptr._version, data._version if data.numel() > 1 else None)


def _matrix_refs(data, indices, indptr):
  return [weakref.ref(indices), weakref.ref(indptr)] + ([weakref.ref(data)] if data.numel() > 1 else [])


def _alive(refs):
  return all(r() is not None for r in refs)


def _set_route(data, indices, indptr, shape, route):
  """Records the kernel family of this matrix ("row", "tiled" or "split"); returns its key."""
  key = _matrix_key(data, indices, indptr, shape[0], shape[1])
  _ROUTES[key] = (_matrix_refs(data, indices, indptr), _versions(data, indices, indptr), route)
  return key


def _route(data, indices, indptr, shape):
  """The autotuned kernel family of this matrix: "row", "tiled", "split", "fixed", or None (not tuned,
  or the arrays changed since)."""
  if not _ROUTES:
    return None
  key = _matrix_key(data, indices, indptr, shape[0], shape[1])
  ent = _ROUTES.get(key)
  if ent is None:
    return None
  refs, ver, route = ent
  if _alive(refs) and ver == _versions(data, indices, indptr):
    return route
  del _ROUTES[key]
  return None


def _plan_kind(data, n, route):
  """Plan kind of an event product: "count" (split plan) for a homogeneous weight on many
  columns, unless the autotuner chose the general plan; "fixed" (fixed-point weights) for
  per-synapse weights unless the autotuner chose the general plan (or the matrix has fewer
  than BPGPU_FIXED_MIN_N columns); "general" otherwise."""
  if data.numel() > 1:
    if route == "fixed" or (route is None and int(n) >= _FIXED_MIN_N):
      return "fixed"
    return "general"
  if route == "tiled":
    return "general"
  if route == "split":
    return "count"
  return "count" if int(n) >= _SPLIT_MIN_N else "general"


def release_plans():
  """Drops every cached plan and autotuned route.  Their device memory is freed once no other
  reference holds the plans (a plan of a 1e6 x 1e6 matrix with fan-out 1000 is about 2.6 GB)."""
  _PLANS.clear()
  _ROUTES.clear()


def plan_cache_bytes():
  """Device bytes held by the cached plans."""
  return sum(int(p.mem.numel()) for _, _, p in _PLANS.values())


def _cached_plan(data, indices, indptr, shape, force=False, routed=True, kind="general"):
  """The plan of this matrix (built on first use), or None when the matrix is below the
  size thresholds, plans are disabled, or the autotuner routed its event product to the row
  kernel.  `force` builds one below the thresholds (an autotuned "tiled"/"split" route, or
  tuning itself); `routed=False` ignores the event product's route (the dense-vector products).
  kind "count" asks for the split plan (homogeneous weights only; other matrices get the
  general plan)."""
  if _PLAN_DISABLE:
    return None
  m, n = int(shape[0]), int(shape[1])
  if not force:
    route = _route(data, indices, indptr, (m, n)) if routed else None
    if route == "row":
      return None
    if route is None and (n < _PLAN_MIN_N or indices.numel() < _PLAN_MIN_NNZ):
      return None
  heter = data.numel() > 1
  if heter and kind == "count":
    kind = "general"
  if not heter and kind == "fixed":
    kind = "general"
  key = (_matrix_key(data, indices, indptr, m, n), kind)
  ver = _versions(data, indices, indptr)
  ent = _PLANS.get(key)
  if ent is not None:
    refs, v, plan = ent
    if _alive(refs) and v == ver:
      return plan
    del _PLANS[key]  # stale: release its memory before building the new plan
  for k in [k for k, (refs, _, _) in _PLANS.items() if not _alive(refs)]:
    del _PLANS[k]
  plan = CSRPlan(indices, indptr, (m, n), data if heter else None, kind=kind)
  _PLANS[key] = (_matrix_refs(data, indices, indptr), ver, plan)
  return plan


def _plan_for(data, indices, indptr, shape):
  """The plan the transposed event product of this matrix runs on (autotuned route first,
  then the size thresholds), or None for the plain CSR kernels."""
  route = _route(data, indices, indptr, shape)
  return _cached_plan(data, indices, indptr, shape, force=route in ("tiled", "split", "fixed"),
                      kind=_plan_kind(data, shape[1], route))


def _valid_choice(choice):
  if choice in ("row", "split", "fixed"):
    return True
  if not isinstance(choice, str) or not choice.startswith("tiled:"):
    return False
  try:
    return int(choice.split(":", 1)[1]) in CSRPlan.variants()
  except ValueError:
    return False


def autotune(data, indices, indptr, events, *, shape: Tuple[int, int], transpose: bool = True,
             reps: int = 10, cache: Optional[tuning.TuneCache] = None, timer=None,
             float_rule=_lib.BP_EV_F32_POS) -> dict:
  """Chooses the kernel family for this matrix at the firing rate of `events` (a spike vector
  representative of the model) and keeps the choice for later ``csrmv`` calls on the same
  arrays: the row-parallel kernel, or the column-tiled plan in one of its compiled variants.

  Every candidate is timed on `events` (``reps`` calls after two warm-up calls, CUDA events)
  unless `cache` (default: the process cache, file-backed when ``BPGPU_TUNE_CACHE`` is set)
  already holds a record for the same device, sizes, weight kind, event type and half-octave
  rate bucket.  Returns the record: ``{"choice": "row" | "tiled:<variant>", "times_us":
  {...}, "rate": r}``.  Every candidate computes the same product (bit for bit with a
  homogeneous weight), so the choice changes speed only.  With ``transpose=False`` only the
  row-parallel family exists and nothing is timed."""
  dev = events.device if isinstance(events, torch.Tensor) and events.is_cuda else default_device()
  d = float_data(data, dev)
  indices = as_tensor(indices, dev)
  indptr = as_tensor(indptr, dev)
  events = as_tensor(events, dev)
  _check_common(d, indices, indptr, events, shape, bool(transpose))
  if index_type(indptr, "indptr") != index_type(indices, "indices"):
    raise ValueError("indices and indptr must have the same integer type.")
  m, n = int(shape[0]), int(shape[1])
  if not transpose:
    return {"choice": "row", "times_us": {}, "rate": None}
  etype, ev = event_type(events, float_rule)
  if etype == _lib.BP_EV_BOOL:
    active = int(ev.sum())
  elif etype == _lib.BP_EV_F32_POS:
    active = int((ev > 0).sum())
  else:
    active = int((ev != 0).sum())
  rate = active / max(m, 1)
  heter = d.numel() > 1
  key = tuning.make_key("event_csrmv_T", torch.cuda.get_device_name(dev), m, n, indices.numel(), heter, etype,
                        tuning.rate_bucket(rate))
  cache = cache if cache is not None else tuning.default_cache()
  rec = cache.lookup(key)
  if rec is not None and not _valid_choice(rec.get("choice")):
    rec = None  # a record from a build with other variants: time again
  if rec is None:
    out = torch.empty(n, dtype=torch.float32, device=dev)
    cands = {"row": lambda: _event_csrmv(d, indices, indptr, events, shape, True, float_rule, out=out, use_plan=False)}
    plan = _cached_plan(d, indices, indptr, (m, n), force=True)
    if plan is not None:
      w = None if plan.heter else d
      for code in CSRPlan.variants():
        def run(code=code):
          plan.variant = code
          return plan.csrmv(events, w, out=out, float_rule=float_rule)
        cands[f"tiled:{code}"] = run
      if not heter and _lib.lib().bp_csr_plan_count_tile(n) > 0:
        split = _cached_plan(d, indices, indptr, (m, n), force=True, kind="count")
        cands["split"] = lambda: split.csrmv(events, d, out=out, float_rule=float_rule)
      if heter:
        fixed = _cached_plan(d, indices, indptr, (m, n), force=True, kind="fixed")
        cands["fixed"] = lambda: fixed.csrmv(events, None, out=out, float_rule=float_rule)
    best, times = tuning.pick(cands, timer or tuning.cuda_timer(reps))
    rec = {"choice": best, "times_us": times, "rate": rate}
    cache.store(key, rec)
    cache.save()
  mkey = _matrix_key(d, indices, indptr, m, n)
  choice = rec["choice"] if not _PLAN_DISABLE else "row"
  route = choice.split(":", 1)[0]
  _set_route(d, indices, indptr, (m, n), route)
  # keep only the plan the chosen family runs on: each holds about 2.6 bytes per stored entry
  keep = {"tiled": "general", "split": "count", "fixed": "fixed"}.get(route)
  for kind in ("general", "count", "fixed"):
    if kind != keep:
      _PLANS.pop((mkey, kind), None)
  if route == "tiled":
    plan = _cached_plan(d, indices, indptr, (m, n), force=True)
    plan.variant = int(choice.split(":", 1)[1])
  elif route == "split":
    _cached_plan(d, indices, indptr, (m, n), force=True, kind="count")
  elif route == "fixed":
    _cached_plan(d, indices, indptr, (m, n), force=True, kind="fixed")
  return rec


def _check_common(data, indices, indptr, events, shape, transpose):
  if data.ndim != 1:
    raise ValueError(f"data should be a scalar or 1D vector. But we got {data.ndim}-D array.")
  if data.shape[0] not in (1, indices.shape[0]):
    raise ValueError("The size of data should be 1 or be consistent with indices."
                     f"But we got {tuple(data.shape)} != {tuple(indices.shape)}, {tuple(data.shape)} != 1.")
  if indices.ndim != 1:
    raise ValueError("indices should be a 1D vector with integer type.")
  if indptr.ndim != 1:
    raise ValueError("indptr should be a 1D vector with integer type.")
  if events.ndim != 1:
    raise ValueError("events should be a 1D vector.")
  if len(shape) != 2:
    raise ValueError("shape should be a length-2 tuple.")
  if transpose:
    if events.shape[0] != shape[0]:
      raise ValueError(f"Shape mismatch, vec ({events.shape[0]},) @ mat {tuple(shape)}.")
  else:
    if events.shape[0] != shape[1]:
      raise ValueError(f"Shape mismatch, mat {tuple(shape)} @ vec ({events.shape[0]},).")
  if indptr.shape[0] != shape[0] + 1:
    raise ValueError(f"indptr should have shape ({shape[0] + 1},), got {tuple(indptr.shape)}.")


def _event_csrmv(data, indices, indptr, events, shape, transpose, float_rule, out=None, use_plan=True):
  dev = events.device if isinstance(events, torch.Tensor) and events.is_cuda else default_device()
  data = float_data(data, dev)
  indices = as_tensor(indices, dev)
  indptr = as_tensor(indptr, dev)
  events = as_tensor(events, dev)
  _check_common(data, indices, indptr, events, shape, bool(transpose))
  itype = index_type(indices, "indices")
  if index_type(indptr, "indptr") != itype:
    raise ValueError("indices and indptr must have the same integer type.")
  etype, ev = event_type(events, float_rule)
  m, n = int(shape[0]), int(shape[1])
  n_out = n if transpose else m
  if transpose and use_plan:
    plan = _plan_for(data, indices, indptr, (m, n))
    if plan is not None:
      return plan.csrmv(events, None if plan.heter else data, out=out, float_rule=float_rule)
  if out is None:
    out = torch.empty(n_out, dtype=torch.float32, device=dev)
  L = _lib.lib()
  ws_bytes = L.bp_event_csrmv_workspace_size(m, n, int(bool(transpose)))
  ws = _lib.workspace(ws_bytes, dev)
  st = L.bp_event_csrmv(_lib.ptr(data), data.shape[0], _lib.ptr(indices), _lib.ptr(indptr), itype,
                        indices.shape[0], _lib.ptr(ev), etype, m, n, int(bool(transpose)), _lib.ptr(out),
                        _lib.ptr(ws), ws_bytes, _lib.stream_handle(dev))
  _lib.check(st, "event.csrmv")
  return out


def csrmv(data: Union[float, torch.Tensor], indices: torch.Tensor, indptr: torch.Tensor,
          events: torch.Tensor, *, shape: Tuple[int, int], transpose: bool = False) -> torch.Tensor:
  """Product of a sparse CSR matrix and a dense event vector.

  Same contract as ``brainpy.math.event.csrmv``: ``data`` is a scalar or an ``(nse,)``
  float32 array, ``indices``/``indptr`` int32 or int64, ``events`` bool or float32 of
  length ``shape[0]`` (transpose) or ``shape[1]``.  A float event counts when it is
  ``> 0`` (the reference's CPU kernels); its value is not multiplied in.
  Returns float32 of length ``shape[1]`` (transpose) or ``shape[0]``.

  Differentiable in ``data`` and in float ``events`` (reverse and forward mode) with the
  reference's rules (brainpy/_src/math/event/_csr_matvec.py:521-551).
  """
  return _dispatch(data, indices, indptr, events, shape, transpose, _lib.BP_EV_F32_POS)


def csrmv_taichi(data, indices, indptr, events, *, shape, transpose=False):
  """``brainpy.math.event.csrmv_taichi``: as :func:`csrmv`, float events count when ``!= 0``."""
  return _dispatch(data, indices, indptr, events, shape, transpose, _lib.BP_EV_F32_NZ)


def _dispatch(data, indices, indptr, events, shape, transpose, float_rule):
  if _grad.wanted(data, events):
    dev = events.device if isinstance(events, torch.Tensor) and events.is_cuda else default_device()
    d = float_data(data, dev)
    ev = as_tensor(events, dev)
    return _grad.EventCSRMV.apply(d, ev, as_tensor(indices, dev), as_tensor(indptr, dev),
                                  (int(shape[0]), int(shape[1])), bool(transpose), float_rule)
  return _event_csrmv(data, indices, indptr, events, shape, transpose, float_rule)


def csrmv_batch(data, indices, indptr, events, *, shape: Tuple[int, int], transpose: bool = False,
                float_rule=_lib.BP_EV_F32_POS) -> torch.Tensor:
  """csrmv mapped over the leading axis of a (B, len) batch of event vectors: (B, out).

  The reference maps its primitive over a batch with a sequential scan of single calls
  (brainpy/_src/math/op_register/utils.py:16-38); here a transpose product on a planned matrix
  runs the whole batch in one launch pair (bp_event_csrmv_planned_batch), and the other
  cases call the single-vector kernels row by row.  Rows are the single-vector results."""
  dev = events.device if isinstance(events, torch.Tensor) and events.is_cuda else default_device()
  events = as_tensor(events, dev)
  if events.ndim != 2:
    raise ValueError(f"events should be a 2D (batch, length) array, got {events.ndim}-D.")
  m, n = int(shape[0]), int(shape[1])
  if _grad.wanted(data, events):
    rows = [_dispatch(data, indices, indptr, events[b], shape, transpose, float_rule) for b in range(events.shape[0])]
    return torch.stack(rows) if rows else torch.empty((0, n if transpose else m), device=dev)
  d = float_data(data, dev)
  indices = as_tensor(indices, dev)
  indptr = as_tensor(indptr, dev)
  if transpose and events.shape[0] > 0:
    _check_common(d, indices, indptr, events[0], shape, True)
    if index_type(indptr, "indptr") != index_type(indices, "indices"):
      raise ValueError("indices and indptr must have the same integer type.")
    plan = _cached_plan(d, indices, indptr, (m, n), force=_route(d, indices, indptr, (m, n)) in ("tiled", "split"))
    if plan is not None:
      return plan.csrmv_batch(events, None if plan.heter else d, float_rule=float_rule)
  out = torch.empty((events.shape[0], n if transpose else m), dtype=torch.float32, device=dev)
  for b in range(events.shape[0]):
    _event_csrmv(d, indices, indptr, events[b], shape, transpose, float_rule, out=out[b])
  return out


def info(events: torch.Tensor):
  """Event indices (ascending, padded with -1) and the event number, as
  ``brainpy.math.event.info``."""
  dev = events.device if isinstance(events, torch.Tensor) and events.is_cuda else default_device()
  events = as_tensor(events, dev)
  if events.ndim != 1:
    raise TypeError("Only support 1D boolean vector.")
  etype, ev = event_type(events, _lib.BP_EV_F32_NZ)
  n = events.shape[0]
  ids = torch.empty(n, dtype=torch.int32, device=dev)
  num = torch.empty(1, dtype=torch.int32, device=dev)
  L = _lib.lib()
  ws_bytes = L.bp_event_info_workspace_size(n)
  ws = _lib.workspace(ws_bytes, dev)
  st = L.bp_event_info(_lib.ptr(ev), etype, n, _lib.ptr(ids), _lib.ptr(num), _lib.ptr(ws), ws_bytes,
                       _lib.stream_handle(dev))
  _lib.check(st, "event.info")
  return ids, num
