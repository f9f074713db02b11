"""E/I COBA LIF networks on GB300: the consumer of the propagation operators.

Mirrors examples/dynamics_simulation/COBA.py:58-109 (EICOBA_PostAlign): LifRefLTC / LifRef
neurons (brainpy/_src/dyn/neurons/lif.py:348-556), Expon conductances with COBA outputs
(dyn/synapses/abstract_models.py:24-134, dyn/outs/outputs.py:16-54), four event-driven
projections E2E, E2I, I2E, I2I aligned post (dyn/projections/align_post.py:149-282), run by
a DSRunner-style loop (brainpy/_src/runners.py:619-665).

Two execution forms:
* ``run(..., method="cluster")``: the whole run inside one persistent launch
  (bp_net_run); the network must fit one thread-block cluster (n <= 16 x 4096).
* ``run(..., method="ops")``: one event.csrmv / jitconn call per projection and one
  neuron-update kernel per step (the per-operator path), optionally captured as a CUDA graph.
A just-in-time network can also be stored (``EINetwork.materialize``): the same connections
generated once into CSR, stepped by the event-driven CSR products.
"""
import ctypes
import math
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import _lib
from .connect import fixed_prob_csr
from .math import event as _event
from .math import jitconn as _jitconn


_MAX_DELAY = 64  # spike-history steps the cluster runner holds in shared memory


def delay_steps(delay, dt):
  """Delay steps of a registered delay entry (brainpy/_src/delay.py:259-264): None -> 0,
  otherwise ceil(delay / dt) in double precision."""
  return 0 if delay is None else int(math.ceil(float(delay) / float(dt)))


class _DevStep:
  """A device-side time index: *step_dev + offset (CUDA-graph replay)."""

  def __init__(self, step_dev, offset):
    self.step_dev, self.offset = step_dev, int(offset)


@dataclass
class LifParams:
  """Parameters of COBA.py's neurons and synapses (defaults: the example's values)."""
  V_rest: float = -60.0
  V_th: float = -50.0
  V_reset: float = -60.0
  tau: float = 20.0
  tau_ref: float = 5.0
  R: float = 1.0
  tau_e: float = 5.0
  tau_i: float = 10.0
  E_e: float = 0.0
  E_i: float = -80.0
  input: float = 20.0
  ltc: bool = True

  def c(self):
    return _lib.LifParams(self.V_rest, self.V_th, self.V_reset, self.tau, self.tau_ref, self.R, self.tau_e,
                          self.tau_i, self.E_e, self.E_i, self.input, int(self.ltc))


def lif_coba_step(params: LifParams, V, ge, gi, t_last, spike, dge, dgi, step: int, dt: float):
  """One neuron-update step in place (torch tensors on the GPU)."""
  dev = V.device
  st = _lib.lib().bp_lif_coba_step(ctypes.byref(params.c()), V.shape[0], _lib.ptr(V), _lib.ptr(ge), _lib.ptr(gi),
                                   _lib.ptr(t_last), _lib.ptr(spike.view(torch.uint8)),
                                   _lib.ptr(dge) if dge is not None else None,
                                   _lib.ptr(dgi) if dgi is not None else None, int(step), float(dt),
                                   _lib.stream_handle(dev))
  _lib.check(st, "lif_coba_step")


def default_net_tile(n):
  """Neurons per CTA of the cluster runner for an n-neuron network: a quarter of the network
  (more CTAs per network shorten a step: measured 231 K steps/s for the 4000-neuron COBA
  example at 1024 against 108 K at 4096), between 1024 and the runner's maximum width."""
  cap = _lib.lib().bp_net_tile_width()
  t = ((n + 3) // 4 + 63) // 64 * 64
  return max(1024, min(cap, t))


class EINetwork:
  """One E/I COBA network: n neurons, [0, n_exc) excitatory, shared LIF parameters.

  Connectivity is either CSR (``indices``/``indptr`` over all n pre-synaptic rows and n
  post-synaptic columns: the union of E2E+E2I rows and I2E+I2I rows, homogeneous weights
  we / wi) or just-in-time (``jitconn=dict(prob=..., seeds=(s_EE, s_EI, s_IE, s_II))``, the
  four EventJitFPHomoLinear projections of BrainPy, outdim_parallel=True).

  ``delay_e`` / ``delay_i`` (ms, or None) are the synaptic delays of the projections leaving
  the excitatory / inhibitory group (FullProjAlignPostMg(delay=...), brainpy/_src/dyn/
  projections/align_post.py:225-272, registered on the group's VarDelay): the rows propagate
  the spikes of ceil(delay / dt) steps before (brainpy/_src/delay.py:259-264, :334-373); dt is
  the step the delays are counted in."""

  def __init__(self, n, n_exc, *, indices=None, indptr=None, we=0.6, wi=6.7, params: Optional[LifParams] = None,
               jitconn=None, device=None, V0=None, net_tile=None, delay_e=None, delay_i=None, dt=0.1):
    self.n, self.n_exc = int(n), int(n_exc)
    # neurons per CTA in the cluster runner (multiple of 64, at most bp_net_tile_width())
    self.net_tile = int(net_tile) if net_tile is not None else None
    self.we, self.wi = float(we), float(wi)
    self.params = params or LifParams()
    self.device = device or torch.device("cuda", torch.cuda.current_device())
    self.jitconn = jitconn
    if jitconn is None:
      if indices is None or indptr is None:
        raise ValueError("either CSR (indices, indptr) or jitconn parameters are required")
      self.indices = indices.to(self.device)
      self.indptr = indptr.to(self.device)
    dev = self.device
    self.V = (torch.as_tensor(V0, dtype=torch.float32, device=dev).clone() if V0 is not None
              else torch.full((n,), self.params.V_rest, device=dev))
    self.ge = torch.zeros(n, device=dev)
    self.gi = torch.zeros(n, device=dev)
    self.t_last = torch.full((n,), -1e7, device=dev)
    self.spike = torch.zeros(n, dtype=torch.bool, device=dev)
    self.t_step = 0
    self._plan = None
    self._split = None
    self._opc = None
    self._pc = None
    # delays in steps and the spike history: step T's spike bits in ring[T mod L]
    self.delay_dt = float(dt)
    self.d_e, self.d_i = delay_steps(delay_e, dt), delay_steps(delay_i, dt)
    self.ring_len = max(self.d_e, self.d_i)
    if self.ring_len > _MAX_DELAY:
      raise ValueError(f"delays of {self.ring_len} steps exceed the {_MAX_DELAY} steps the runner holds")
    self.words = (self.n + 31) // 32
    self.ring = (torch.zeros((self.ring_len, self.words), dtype=torch.int32, device=dev) if self.ring_len else None)

  # ---- construction helpers ---------------------------------------------------------
  @classmethod
  def fixed_prob(cls, n_exc, n_inh, prob=0.02, we=0.6, wi=6.7, seed=0, params=None, device=None, V0=None,
                 net_tile=None, delay_e=None, delay_i=None, dt=0.1):
    """COBA.py's four FixedProb(prob) projections with fan-out int(post*prob) per group,
    merged into one n x n CSR (E rows: E targets then I targets; I rows likewise)."""
    dev = device or torch.device("cuda", torch.cuda.current_device())
    n = n_exc + n_inh
    blocks = []
    for g, (rows, seed_off) in enumerate(((n_exc, 0), (n_inh, 2))):
      i_ee, _ = fixed_prob_csr(rows, n_exc, int(n_exc * prob), seed=seed * 4 + seed_off, device=dev)
      i_ei, _ = fixed_prob_csr(rows, n_inh, int(n_inh * prob), seed=seed * 4 + seed_off + 1, device=dev)
      ke, ki = int(n_exc * prob), int(n_inh * prob)
      row_idx = torch.cat([i_ee.view(rows, ke), i_ei.view(rows, ki) + n_exc], dim=1) if rows else i_ee.view(0, ke + ki)
      blocks.append(row_idx.reshape(-1))
    k_row = int(n_exc * prob) + int(n_inh * prob)
    indices = torch.cat(blocks).to(torch.int32)
    indptr = (torch.arange(n + 1, device=dev, dtype=torch.int64) * k_row).to(torch.int32)
    return cls(n, n_exc, indices=indices, indptr=indptr, we=we, wi=wi, params=params, device=dev, V0=V0,
               net_tile=net_tile, delay_e=delay_e, delay_i=delay_i, dt=dt)

  def materialize(self, index_dtype=None):
    """This just-in-time network with its connectivity stored: a CSR network with the same
    neurons, weights, delays and state whose row j holds the postsynaptic neurons that the four
    pull projections (outdim_parallel=True) connect presynaptic neuron j to, generated once
    from the same streams (bp_jitconn_csr) instead of on every step.  Its steps are the
    event-driven CSR products; with homogeneous weights both forms add exact event counts
    times w, so the two networks spike alike, step for step.  The indices are int32 while
    they fit (about 2e9 synapses), int64 beyond (or as `index_dtype` asks)."""
    if self.jitconn is None:
      raise ValueError("the network's connectivity is already stored")
    if not bool(self.jitconn.get("outdim_parallel", True)):
      raise ValueError("materialize takes the pull form (outdim_parallel=True); the push form runs on the "
                       "whole-GPU runner")
    L = _lib.lib()
    dev, sp = self.device, _lib.stream_handle(self.device)
    ne, n = self.n_exc, self.n
    ni = n - ne
    clen = _jitconn.conn_len(self.jitconn["prob"])
    seeds = [_jitconn._seed(x, False) for x in self.jitconn["seeds"]]
    # (outputs, inputs, seed, output offset): E2E, E2I from the excitatory rows, I2E, I2I from the
    # inhibitory rows, as _propagate_ops calls them
    projs = ((ne, ne, seeds[0], 0), (ni, ne, seeds[1], ne), (ne, ni, seeds[2], 0), (ni, ni, seeds[3], ne))
    counts = []
    for n_out, n_in, sd, _ in projs:
      c = torch.zeros(max(n_in, 1), dtype=torch.int32, device=dev)
      _lib.check(L.bp_jitconn_csr(0, clen, sd, n_out, n_in, _lib.ptr(c), None, 0, None, 0, _lib.BP_I32, sp),
                 "jitconn_csr")
      counts.append(c[:n_in].to(torch.int64))
    row_len = torch.cat([counts[0] + counts[1], counts[2] + counts[3]])
    indptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    torch.cumsum(row_len, 0, out=indptr[1:])
    nnz = int(indptr[-1])
    if index_dtype is None:
      index_dtype = torch.int32 if nnz < 2 ** 31 - 1 else torch.int64
    itype = _lib.BP_I32 if index_dtype == torch.int32 else _lib.BP_I64
    indices = torch.empty(max(nnz, 1), dtype=index_dtype, device=dev)
    bases = (indptr[:ne], indptr[:ne] + counts[0], indptr[ne:n], indptr[ne:n] + counts[2])
    for (n_out, n_in, sd, off), base in zip(projs, bases):
      base = base.contiguous()
      _lib.check(L.bp_jitconn_csr(1, clen, sd, n_out, n_in, None, _lib.ptr(base), off, _lib.ptr(indices), nnz, itype,
                                  sp), "jitconn_csr")
    net = EINetwork(n, ne, indices=indices[:nnz], indptr=indptr.to(index_dtype), we=self.we, wi=self.wi,
                    params=self.params, device=dev, V0=self.V, net_tile=self.net_tile, dt=self.delay_dt)
    net.reset_state(self.V, self.ge, self.gi, self.t_last, self.spike, self.t_step)
    # the same delays (in steps) and spike history
    net.d_e, net.d_i, net.ring_len = self.d_e, self.d_i, self.ring_len
    net.ring = self.ring.clone() if self.ring is not None else None
    return net

  def reset_state(self, V, ge, gi, t_last, spike, t_step=0):
    """Overwrites the state (tensors of length n) and the time index."""
    self.V.copy_(V)
    self.ge.copy_(ge)
    self.gi.copy_(gi)
    self.t_last.copy_(t_last)
    self.spike.copy_(spike)
    self.t_step = int(t_step)
    if self.ring is not None:
      self.ring.zero_()  # VarDelay.reset_state: the history starts at zero

  def state_numpy(self):
    return {"V": self.V.cpu().numpy(), "ge": self.ge.cpu().numpy(), "gi": self.gi.cpu().numpy(),
            "t_last": self.t_last.cpu().numpy(), "spike": self.spike.cpu().numpy().astype(np.uint8)}

  # ---- persistent cluster form --------------------------------------------------------
  def _cluster_plan(self):
    if self._plan is None:
      tw = self.net_tile or default_net_tile(self.n)
      if tw % 64 or not 64 <= tw <= _lib.lib().bp_net_tile_width():
        raise ValueError(f"net_tile {tw} must be a multiple of 64 in [64, {_lib.lib().bp_net_tile_width()}]")
      self._plan = _event.CSRPlan(self.indices, self.indptr, (self.n, self.n), tile_w=tw, cluster=1)
      if self._plan.c.n_tiles > _lib.lib().bp_net_max_tiles():
        raise ValueError(f"network of {self.n} neurons exceeds one cluster ({_lib.lib().bp_net_max_tiles()} tiles)")
    return self._plan

  def descriptor(self, spike_counts=None, raster=None, v_trace=None, trace_steps=0, step_limit=0, plan=None):
    plan = plan if plan is not None else self._cluster_plan()
    so, idx, w = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    _lib.check(_lib.lib().bp_csr_plan_arrays(ctypes.byref(plan.c), ctypes.byref(so), ctypes.byref(idx),
                                             ctypes.byref(w)), "csr_plan_arrays")
    d = _lib.NetDesc()
    d.n, d.n_exc = self.n, self.n_exc
    d.tile_w, d.n_tiles = plan.tile_w, plan.c.n_tiles
    d.seg_off, d.idx = so, idx
    d.we, d.wi = self.we, self.wi
    d.p = self.params.c()
    d.V, d.ge, d.gi, d.t_last = (self.V.data_ptr(), self.ge.data_ptr(), self.gi.data_ptr(), self.t_last.data_ptr())
    d.spike = self.spike.data_ptr()
    d.spike_counts = spike_counts.data_ptr() if spike_counts is not None else None
    d.raster = raster.data_ptr() if raster is not None else None
    d.v_trace = v_trace.data_ptr() if v_trace is not None else None
    d.trace_steps = int(trace_steps)
    d.step_limit = int(step_limit)
    d.step0 = int(self.t_step)
    d.delay_e, d.delay_i, d.ring_len = self.d_e, self.d_i, self.ring_len
    d.ring = self.ring.data_ptr() if self.ring is not None else None
    return d

  def fits_cluster(self):
    """Whether the cluster runner (one thread-block cluster per network) can hold the network."""
    L = _lib.lib()
    return self.jitconn is None and self.n <= L.bp_net_max_tiles() * L.bp_net_tile_width()

  # ---- whole-GPU persistent form (networks larger than a cluster) ----------------------
  def grid_eligible(self):
    """Whether the network can run in one persistent launch over the GPU: CSR connectivity
    (bp_net_run_grid) with every tile's cluster resident at once and no column with 65,536
    or more incoming entries (the runner counts excitatory and inhibitory events in the two
    16-bit halves of one word); or just-in-time connectivity in the push form
    (outdim_parallel=False; bp_net_run_grid_jit) without delays."""
    if self.jitconn is not None:
      return (not bool(self.jitconn.get("outdim_parallel", True)) and self.ring is None
              and self.n * 32 < 2 ** 31)
    if _lib.lib().bp_net_grid_tile(self.n) <= 0:
      return False
    if not hasattr(self, "_indeg_ok"):
      deg = torch.bincount(self.indices.to(torch.int64), minlength=self.n)
      self._indeg_ok = bool(int(deg.max()) < 65536) if deg.numel() else True
    return self._indeg_ok

  def _grid_state(self):
    """The runner's plan (tiles of bp_net_grid_tile(n) columns) and workspace, built once
    (just-in-time networks: the workspace only)."""
    if getattr(self, "_grid", None) is None and self.jitconn is not None:
      if not self.grid_eligible():
        raise ValueError("the whole-GPU runner takes just-in-time networks in the push form (outdim_parallel="
                         "False) without delays")
      nb = int(_lib.lib().bp_net_grid_jit_workspace_size(self.n))
      self._grid = (None, torch.zeros(max(nb, 1), dtype=torch.uint8, device=self.device))
    if getattr(self, "_grid", None) is None:
      if not self.grid_eligible():
        raise ValueError(f"network of {self.n} neurons cannot run on the grid runner (jitconn, too many tiles "
                         "for the resident clusters, or a column with 65,536 or more inputs)")
      L = _lib.lib()
      tw = int(L.bp_net_grid_tile(self.n))
      plan = _event.CSRPlan(self.indices, self.indptr, (self.n, self.n), tile_w=tw, cluster=1)
      ws = torch.zeros(max(int(L.bp_net_grid_workspace_size(self.n, tw)), 1), dtype=torch.uint8, device=self.device)
      self._grid = (plan, ws)
    return self._grid

  def _run_grid(self, steps, dt, counts, trace, trace_steps):
    plan, ws = self._grid_state()
    if self.jitconn is not None:
      d = self._state_desc(counts, trace, trace_steps)
      seeds = (ctypes.c_uint32 * 4)(*[_jitconn._seed(x, False) for x in self.jitconn["seeds"]])
      st = _lib.lib().bp_net_run_grid_jit(ctypes.byref(d), seeds, _jitconn.conn_len(self.jitconn["prob"]), 0,
                                          int(steps), float(dt), _lib.ptr(ws), ws.numel(),
                                          _lib.stream_handle(self.device))
      _lib.check(st, "net_run_grid_jit")
      self.t_step += steps
      return
    d = self.descriptor(counts, None, trace, trace_steps, 0, plan=plan)
    st = _lib.lib().bp_net_run_grid(ctypes.byref(d), 0, int(steps), float(dt), _lib.ptr(ws), ws.numel(),
                                    _lib.stream_handle(self.device))
    _lib.check(st, "net_run_grid")
    self.t_step += steps

  def _state_desc(self, spike_counts=None, v_trace=None, trace_steps=0):
    """A descriptor of the state and parameters only (no connectivity plan)."""
    d = _lib.NetDesc()
    d.n, d.n_exc = self.n, self.n_exc
    d.we, d.wi = self.we, self.wi
    d.p = self.params.c()
    d.V, d.ge, d.gi, d.t_last = (self.V.data_ptr(), self.ge.data_ptr(), self.gi.data_ptr(), self.t_last.data_ptr())
    d.spike = self.spike.data_ptr()
    d.spike_counts = spike_counts.data_ptr() if spike_counts is not None else None
    d.v_trace = v_trace.data_ptr() if v_trace is not None else None
    d.trace_steps = int(trace_steps)
    d.step0 = int(self.t_step)
    return d

  def grid_error(self):
    """The grid runner's error word over every run of this network (0: every barrier wait
    ended); waits for the runs."""
    if getattr(self, "_grid", None) is None:
      return 0
    err = ctypes.c_int32(0)
    _lib.check(_lib.lib().bp_net_grid_error(_lib.ptr(self._grid[1]), ctypes.byref(err),
                                            _lib.stream_handle(self.device)), "net_grid_error")
    return int(err.value)

  # ---- per-operator form ------------------------------------------------------------
  def _csr_split(self):
    """Views of the merged CSR as an excitatory-row and an inhibitory-row matrix."""
    if self._split is None:
      ne = self.n_exc
      ptr = self.indptr.to(torch.int64)
      e_end = int(ptr[ne])
      exc = (self.indices[:e_end], self.indptr[: ne + 1])
      inh = (self.indices[e_end:], (self.indptr[ne:].to(torch.int64) - e_end).to(self.indptr.dtype))
      self._split = (exc, inh)
    return self._split

  def _delayed_spikes(self, T):
    """(excitatory, inhibitory) spike vectors the projections of step T read: self.spike
    when the group has no delay, otherwise the history slot of step T - d.  T is an int or a
    _DevStep (CUDA-graph replay)."""
    ne = self.n_exc
    if not hasattr(self, "_dspk"):
      self._dspk = torch.zeros(self.n, dtype=torch.bool, device=self.device)
    step, sdev = (T.offset, T.step_dev) if isinstance(T, _DevStep) else (int(T), None)
    out = []
    for d, lo, hi in ((self.d_e, 0, ne), (self.d_i, ne, self.n)):
      if d == 0:
        out.append(self.spike[lo:hi])
        continue
      dst = self._dspk[lo:hi]
      st = _lib.lib().bp_spike_ring_read(_lib.ptr(self.ring), self.ring_len, self.n, lo, hi - lo, d, step,
                                         _lib.ptr(sdev) if sdev is not None else None,
                                         _lib.ptr(dst.view(torch.uint8)), _lib.stream_handle(self.device))
      _lib.check(st, "spike_ring_read")
      out.append(dst)
    return out

  def _record_spikes(self, T):
    """Stores self.spike as step T's history slot."""
    if self.ring is None:
      return
    step, sdev = (T.offset, T.step_dev) if isinstance(T, _DevStep) else (int(T), None)
    st = _lib.lib().bp_spike_ring_record(_lib.ptr(self.spike.view(torch.uint8)), self.n, _lib.ptr(self.ring),
                                         self.ring_len, step, _lib.ptr(sdev) if sdev is not None else None,
                                         _lib.stream_handle(self.device))
    _lib.check(st, "spike_ring_record")

  def _csr_ops(self):
    """Call state of the two event.csrmv projections of the per-operator path, built once.
    For the excitatory-row and the inhibitory-row matrix: its weight as a device scalar, a
    persistent output vector, and either the plan that event.csrmv runs on for this matrix
    (large networks) or the argument list of a direct bp_event_csrmv call with its workspace
    (small ones, where the library runs a single-launch kernel).  The checks and allocations
    of the public call are done here once instead of every step; the result is the same."""
    if self._opc is None:
      n = self.n
      L = _lib.lib()
      ops = []
      # the weights as device scalars, kept for the network's life: an autotuned route is keyed
      # by the arrays of the product, these included
      if getattr(self, "_wts", None) is None:
        self._wts = tuple(torch.full((1,), w, device=self.device) for w in (self.we, self.wi))
      for (ind, ptr), m, wt in zip(self._csr_split(), (self.n_exc, n - self.n_exc), self._wts):
        out = torch.empty(n, device=self.device)
        plan = _event._plan_for(wt, ind, ptr, (m, n))
        ws, args = None, None
        if plan is None:
          wsb = int(L.bp_event_csrmv_workspace_size(m, n, 1))
          ws = _lib.workspace(wsb, self.device)
          itype = _lib.BP_I32 if ind.dtype == torch.int32 else _lib.BP_I64
          args = (wt.data_ptr(), ind.data_ptr() if ind.numel() else 0, ptr.data_ptr(), itype, ind.numel(), m, n,
                  out.data_ptr(), ws.data_ptr(), wsb)
        ops.append((wt, out, plan, ws, args))
      self._opc = ops
    return self._opc

  def tune_ops(self, spikes=None):
    """Autotunes the per-operator path's two event products (event.autotune: row-parallel
    kernel, the tiled plan's variants, the counting plan) on the rows' spikes of `spikes`
    (default: the network's current spikes, so run it into its firing regime first).  Later
    steps use the chosen kernels; every choice gives the same result bit for bit.  Returns
    the two tuning records (excitatory rows, inhibitory rows)."""
    if self.jitconn is not None:
      raise ValueError("tune_ops tunes the CSR products of a network with stored connectivity")
    sp = self.spike if spikes is None else spikes
    ne, n = self.n_exc, self.n
    self._csr_ops()
    recs = [_event.autotune(wt, ind, ptr, ev, shape=(m, n))
            for wt, (ind, ptr), m, ev in zip(self._wts, self._csr_split(), (ne, n - ne), (sp[:ne], sp[ne:]))]
    self._opc = None  # rebuilt on the tuned routes
    if hasattr(self, "_graph"):
      del self._graph
    return recs

  def _propagate_ops(self, T=None):
    """Conductance increments of one step (per-operator path): the rows' spikes of the
    previous step, or of their group's delay before step T."""
    ne, n = self.n_exc, self.n
    se, si = (self.spike[:ne], self.spike[ne:]) if self.ring is None else self._delayed_spikes(T)
    if self.jitconn is None:
      res = []
      fn = None
      for (wt, out, plan, _, args), ev in zip(self._csr_ops(), (se, si)):
        if plan is not None:
          res.append(plan.csrmv(ev, wt, out=out))
          continue
        if fn is None:
          fn, sp = _lib.lib().bp_event_csrmv, _lib.raw_stream(self.device)
        w, ix, ip, itype, nnz, m, nn, o, ws, wsb = args
        st = fn(w, 1, ix, ip, itype, nnz, ev.data_ptr(), _lib.BP_EV_BOOL, m, nn, 1, o, ws, wsb, sp)
        if st:
          _lib.check(st, "event.csrmv")
        res.append(out)
      return res[0], res[1]
    p, s = self.jitconn["prob"], self.jitconn["seeds"]
    odp = bool(self.jitconn.get("outdim_parallel", True))
    ni = n - ne
    dge = torch.empty(n, device=self.device)
    dgi = torch.empty(n, device=self.device)
    # EventJitFPHomoLinear(num_in, num_out, atomic=not odp): shape=(num_out, num_in)
    _jitconn._mv("homo", True, se, self.we, 0.0, p, s[0], (ne, ne), False, odp, False, out=dge[:ne])
    _jitconn._mv("homo", True, se, self.we, 0.0, p, s[1], (ni, ne), False, odp, False, out=dge[ne:])
    _jitconn._mv("homo", True, si, self.wi, 0.0, p, s[2], (ne, ni), False, odp, False, out=dgi[:ne])
    _jitconn._mv("homo", True, si, self.wi, 0.0, p, s[3], (ni, ni), False, odp, False, out=dgi[ne:])
    return dge, dgi

  def step_ops(self, dt, step_dev=None, offset=0):
    """One step through the per-operator path (propagation calls + neuron kernel)."""
    T = self.t_step if step_dev is None else _DevStep(step_dev, offset)
    dge, dgi = self._propagate_ops(T)
    pc = self._pc if self._pc is not None else ctypes.byref(self.params.c())
    if step_dev is None:
      st = _lib.lib().bp_lif_coba_step(pc, self.n, self.V.data_ptr(), self.ge.data_ptr(), self.gi.data_ptr(),
                                       self.t_last.data_ptr(), self.spike.data_ptr(), dge.data_ptr(),
                                       dgi.data_ptr(), int(self.t_step), float(dt), _lib.raw_stream(self.device))
      if st:
        _lib.check(st, "lif_coba_step")
      self._record_spikes(T)
      self.t_step += 1
      return
    st = _lib.lib().bp_lif_coba_step_dev(pc, self.n, _lib.ptr(self.V), _lib.ptr(self.ge),
                                         _lib.ptr(self.gi), _lib.ptr(self.t_last),
                                         _lib.ptr(self.spike.view(torch.uint8)), _lib.ptr(dge), _lib.ptr(dgi),
                                         _lib.ptr(step_dev), int(offset), float(dt), _lib.stream_handle(self.device))
    _lib.check(st, "lif_coba_step_dev")
    self._record_spikes(T)

  def run(self, steps, dt=0.1, method="cluster", spike_counts=None, v_trace_steps=0, graph_steps=0):
    """Advances `steps` steps.  Returns (spike counts per step [steps] int32, V trace or None).
    method "cluster": one persistent launch, on one thread-block cluster when the network
    fits one (n <= 16 x 4096), otherwise over the whole GPU (bp_net_run_grid; see
    ``grid_eligible``); "grid": the whole-GPU runner; "ops": per-operator launches, replayed
    from a CUDA graph of `graph_steps` steps when graph_steps > 0."""
    counts = spike_counts if spike_counts is not None else torch.zeros(steps, dtype=torch.int32, device=self.device)
    if self.ring is not None and abs(float(dt) - self.delay_dt) > 1e-12:
      raise ValueError(f"the delays were counted in steps of dt={self.delay_dt}; run with that dt, not {dt}")
    if method == "cluster" and not self.fits_cluster():
      method = "grid"
    if method == "grid":
      trace = torch.empty((v_trace_steps, self.n), device=self.device) if v_trace_steps else None
      self._run_grid(steps, dt, counts, trace, v_trace_steps)
      return counts, trace
    if method == "cluster":
      trace = torch.empty((v_trace_steps, self.n), device=self.device) if v_trace_steps else None
      run_networks([self], steps, dt, spike_counts=[counts], v_traces=[trace] if trace is not None else None,
                   trace_steps=v_trace_steps)
      return counts, trace
    if method != "ops":
      raise ValueError(f"unknown method {method!r}")
    if graph_steps:
      self._run_ops_graph(steps, dt, counts, graph_steps)
      return counts, None
    trace = []
    self._pc = ctypes.byref(self.params.c())  # the parameters stay fixed during a run
    try:
      for s in range(steps):
        self.step_ops(dt)
        if counts.dtype == torch.int32:
          torch.sum(self.spike, 0, dtype=torch.int32, out=counts[s])
        else:
          counts[s] = self.spike.sum()
        if s < v_trace_steps:
          trace.append(self.V.clone())
    finally:
      self._pc = None
    return counts, (torch.stack(trace) if trace else None)

  def _run_ops_graph(self, steps, dt, counts, graph_steps):
    """Per-operator steps replayed from one captured CUDA graph of `graph_steps` steps; the
    time index comes from device memory so the same graph serves every block of steps."""
    done = 0
    if not hasattr(self, "_graph") and steps > 0:
      self.step_ops(dt)  # warm-up outside capture: plans, workspaces, cached weights
      counts[0] = self.spike.sum()
      done = 1
    if not hasattr(self, "_graph") or self._graph[0] != graph_steps:
      step_dev = torch.zeros(1, dtype=torch.int32, device=self.device)
      buf = torch.zeros(graph_steps, dtype=torch.int32, device=self.device)
      g = torch.cuda.CUDAGraph()
      torch.cuda.synchronize()
      # thread_local: another host thread (a server's job builder) may allocate while this
      # thread captures; only this thread's calls are checked for capture safety
      with torch.cuda.graph(g, capture_error_mode="thread_local"):
        for j in range(graph_steps):
          self.step_ops(dt, step_dev=step_dev, offset=j)
          buf[j] = self.spike.sum()
      self._graph = (graph_steps, g, step_dev, buf)
    _, g, step_dev, buf = self._graph
    while steps - done >= graph_steps:
      step_dev.fill_(self.t_step)
      g.replay()
      counts[done:done + graph_steps] = buf
      self.t_step += graph_steps
      done += graph_steps
    while done < steps:
      self.step_ops(dt)
      counts[done] = self.spike.sum()
      done += 1
    return counts


class NetBatch:
  """A fixed set of networks simulated together by the persistent cluster runner: one launch
  per cluster size (networks of one size run concurrently, one cluster each, each at its own
  time index and step limit), the launches of the different sizes concurrent on side streams
  forked from the current stream and joined back to it.

  The descriptors live in device buffers that are rewritten (from pinned host memory, on the
  current stream) before every run, so the launches can be captured once as a CUDA graph
  (``capture``) and the whole batch then advances by one graph launch per ``replay``: every
  replay continues each network from its current time index, with new spike-count outputs
  and step limits.  Results do not depend on the form."""

  def __init__(self, nets, dt=0.1, concurrent=True):
    self.nets = list(nets)
    self.dt = float(dt)
    self.dev = self.nets[0].device if self.nets else None
    groups = {}
    for k, net in enumerate(self.nets):
      groups.setdefault(net.descriptor().n_tiles, []).append(k)
    # largest launches (CTAs) first: they set the run's length
    self.groups = sorted(groups.items(), key=lambda kv: (-kv[0] * len(kv[1]), kv[0]))
    sz = ctypes.sizeof(_lib.NetDesc)
    self._desc = [torch.empty(len(ix) * sz, dtype=torch.uint8, device=self.dev) for _, ix in self.groups]
    self.concurrent = bool(concurrent)
    self._graph = None

  @property
  def launches(self):
    return len(self.groups)

  def _write(self, spike_counts, step_limits, v_traces, trace_steps):
    for (_, ix), dbuf in zip(self.groups, self._desc):
      arr = (_lib.NetDesc * len(ix))(*[
          self.nets[k].descriptor(spike_counts[k] if spike_counts else None, None,
                                  v_traces[k] if v_traces else None, trace_steps,
                                  int(step_limits[k]) if step_limits is not None else 0) for k in ix])
      host = torch.empty(dbuf.numel(), dtype=torch.uint8, pin_memory=True)
      ctypes.memmove(host.data_ptr(), ctypes.addressof(arr), ctypes.sizeof(arr))
      dbuf.copy_(host, non_blocking=True)  # the pinned block is reused only after the copy

  def _launches(self, steps):
    L = _lib.lib()
    cur = torch.cuda.current_stream(self.dev)
    streams = _side_streams(self.dev, len(self.groups)) if self.concurrent and len(self.groups) > 1 else [cur]
    for s in streams:
      if s is not cur:
        s.wait_stream(cur)
    for (cl, ix), dbuf, s in zip(self.groups, self._desc, streams * len(self.groups)):
      with torch.cuda.stream(s):
        st = L.bp_net_run(_lib.ptr(dbuf), len(ix), cl, 0, int(steps), self.dt, _lib.stream_handle(self.dev))
      _lib.check(st, "net_run")
    for s in streams:
      if s is not cur:
        cur.wait_stream(s)

  def _advance(self, steps, step_limits):
    for k, net in enumerate(self.nets):
      lim = int(step_limits[k]) if step_limits is not None else 0
      net.t_step += min(steps, lim) if lim > 0 else steps

  def run(self, steps, spike_counts=None, step_limits=None, v_traces=None, trace_steps=0):
    """Advances every network by `steps` steps (or its step limit)."""
    if not self.nets or steps <= 0:
      return
    self._write(spike_counts, step_limits, v_traces, trace_steps)
    self._launches(steps)
    self._advance(steps, step_limits)

  def capture(self, steps):
    """Captures the launches of a `steps`-step run as one CUDA graph (nothing runs)."""
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize(self.dev)
    with torch.cuda.graph(g, capture_error_mode="thread_local"):
      self._launches(steps)
    self._graph = (int(steps), g)
    return g

  def replay(self, spike_counts=None, step_limits=None):
    """One launch of the captured graph: every network advances by the captured number of
    steps (or its step limit), from its current time index."""
    if self._graph is None:
      raise RuntimeError("capture() the batch first")
    steps, g = self._graph
    self._write(spike_counts, step_limits, None, 0)
    g.replay()
    self._advance(steps, step_limits)


_SIDE_STREAMS = {}  # device index -> side streams of the batched runner


def _side_streams(dev, k):
  idx = dev.index if dev.index is not None else torch.cuda.current_device()
  pool = _SIDE_STREAMS.setdefault(idx, [])
  while len(pool) < k:
    pool.append(torch.cuda.Stream(device=dev))
  return pool[:k]


def run_networks(nets, steps, dt=0.1, spike_counts=None, v_traces=None, trace_steps=0, step_limits=None,
                 concurrent=True):
  """Runs every network for `steps` steps (or its own step limit) in persistent cluster
  launches (a one-off NetBatch): one launch per cluster size, networks of one size
  concurrently, one cluster each, each at its own time index.  With `concurrent`, the
  launches of the different sizes run concurrently on side streams; results do not depend
  on it.  Returns the batch (its descriptor buffers stay valid while it is held)."""
  if not nets:
    return None
  b = NetBatch(nets, dt, concurrent=concurrent)
  b.run(steps, spike_counts=spike_counts, step_limits=step_limits, v_traces=v_traces, trace_steps=trace_steps)
  return b


def tile_candidates(n, candidates=(1024, 2048, 4096)):
  """Neurons per CTA of the cluster runner that an n-neuron network can take: multiples of 64
  within the runner's width, with at most the runner's maximum of CTAs per cluster."""
  L = _lib.lib()
  cap, tmax = L.bp_net_tile_width(), L.bp_net_max_tiles()
  return [int(t) for t in candidates if t % 64 == 0 and 64 <= t <= cap and -(-int(n) // int(t)) <= tmax]


def size_class(n):
  """Half-octave size class of a network (round(2 log2 n) / 2): the unit of tile tuning."""
  return round(2.0 * math.log2(max(int(n), 1))) / 2.0


def autotune_net_tiles(nets, candidates=(1024, 2048, 4096), steps=100, cache=None):
  """Chooses the cluster runner's neurons per CTA (and so the cluster shape, ceil(n / tile)
  CTAs) for every network, per half-octave size class, and applies it (the networks' runner
  plans are rebuilt on next use).

  A class is timed on its median network: for each candidate tile, a copy of that network
  (same connectivity, parameters and state) runs `steps` steps alone after a warm-up; the
  choice minimises the device time a network-step takes from the GPU, the step time times
  the CTAs it holds, which is what the throughput of a batch that fills the GPU depends on.
  Choices are kept in the tuning cache (``tuning.default_cache()`` unless one is given) under
  the device and class, so later batches and processes apply them without timing.  Results
  do not depend on the tile.  Returns {class: record}."""
  from . import tuning
  cache = cache if cache is not None else tuning.default_cache()
  classes = {}
  for net in nets:
    if net.jitconn is None:
      classes.setdefault(size_class(net.n), []).append(net)
  out = {}
  for cls, members in sorted(classes.items()):
    n_max = max(m.n for m in members)
    cands = tile_candidates(n_max, candidates)
    if not cands:
      continue
    dev = members[0].device
    key = f"net_tile|{torch.cuda.get_device_name(dev)}|class={cls:+.1f}|cands={','.join(map(str, cands))}"
    rec = cache.lookup(key)
    if rec is None or int(rec.get("choice", -1)) not in cands:
      rep = sorted(members, key=lambda m: m.n)[len(members) // 2]
      cost, per_step = {}, {}
      for t in cands:
        probe = EINetwork(rep.n, rep.n_exc, indices=rep.indices, indptr=rep.indptr, we=rep.we, wi=rep.wi,
                          params=rep.params, device=dev, V0=rep.V, net_tile=t)
        probe.run(max(steps // 4, 1))  # plan build, module load, firing under way
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        probe.run(steps)
        t1.record()
        t1.synchronize()
        us = t0.elapsed_time(t1) * 1e3 / steps
        per_step[str(t)] = us
        cost[str(t)] = us * (-(-rep.n // t))
        del probe
      best = min(cands, key=lambda t: (cost[str(t)], -t))
      rec = {"choice": int(best), "cta_us_per_step": cost, "us_per_step": per_step, "timed_on_n": int(rep.n)}
      cache.store(key, rec)
      cache.save()
    best = int(rec["choice"])
    for m in members:
      if m.net_tile != best:
        m.net_tile = best
        m._plan = None
    out[cls] = rec
  return out
