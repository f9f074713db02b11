"""The synaptic-projection layers that call the propagation operators, as in
brainpy/_src/dnn/linear.py: CSRLinear / EventCSRLinear (:490-649) and
JitFP{Homo,Uniform,Normal}Linear / EventJitFP{Homo,Uniform,Normal}Linear (:805-1280).

Same constructor arguments and `update` semantics: CSR layers take the connection's
(indices, indptr) -- from `conn.require('csr')` when given a BrainPy-style connector -- with
shape (pre_num, post_num) and transpose=True by default; just-in-time layers use
shape=(num_out, num_in) and outdim_parallel = not atomic.  Inputs of more than one dimension
are treated as a batch of vectors along the last axis (one launch pair for a planned CSR
product).  Weights given as tensors that require a gradient are trained through the operators'
differentiation rules.  The CSR layers' STDP updates (`stdp_update`, `csr_on_pre_update`,
`csc_on_post_update`, linear.py:517-543 and :650-698) are here; sharding is not part of this
package.
"""
from typing import Optional

import numpy as np
import torch

from .math import event as _event
from .math import jitconn as _jitconn
from .math import sparse as _sparse
from . import _lib
from .math._utils import as_tensor, default_device, index_type

__all__ = ["CSRLinear", "EventCSRLinear", "JitFPHomoLinear", "JitFPUniformLinear", "JitFPNormalLinear",
           "EventJitFPHomoLinear", "EventJitFPUniformLinear", "EventJitFPNormalLinear",
           "csr_on_pre_update", "csc_on_post_update"]


def _batched(fn, x, batch_fn=None):
  """fn over the last axis of x (fn takes and returns 1-D tensors); batch_fn, when given,
  maps a (B, len) batch in one call."""
  if x.ndim == 1:
    return fn(x)
  if x.ndim == 0:
    raise ValueError("the input must have at least one dimension")
  lead = x.shape[:-1]
  flat = x.reshape(-1, x.shape[-1])
  if batch_fn is not None:
    y = batch_fn(flat)
  else:
    ys = [fn(flat[b]) for b in range(flat.shape[0])]
    y = torch.stack(ys) if ys else torch.empty((0, 0), dtype=torch.float32, device=x.device)
  return y.reshape(tuple(lead) + (y.shape[-1],))


def _spike_arg(spike, dev):
  sp = as_tensor(spike, dev)
  if sp.dtype == torch.bool:
    return _lib.BP_EV_BOOL, sp.view(torch.uint8)
  if sp.dtype != torch.float32:
    sp = sp.to(torch.float32)
  return _lib.BP_EV_F32_NZ, sp


def _bounds(w_min, w_max):
  return (-np.inf if w_min is None else float(w_min)), (np.inf if w_max is None else float(w_max))


_STDP_WS = {}


def _stdp_workspace(rows, dev):
  """One compaction workspace per (device, stream), grown on demand; calls on one stream are
  ordered, so they can share it."""
  key = (dev.index, _lib.raw_stream(dev))
  need = _lib.lib().bp_stdp_workspace_size(rows)
  ws = _STDP_WS.get(key)
  if ws is None or ws.numel() < need:
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    _STDP_WS[key] = ws
  return ws


def _plastic(name, w, out, spike, trace, w_min, w_max, rows, call):
  dev = w.device if isinstance(w, torch.Tensor) and w.is_cuda else default_device()
  w = as_tensor(w, dev)
  if w.dtype != torch.float32 or w.ndim != 1:
    raise ValueError(f"{name}: the weight must be a 1D float32 array, got {w.dtype} {tuple(w.shape)}")
  if out is None:
    out = torch.empty_like(w)
  et, sp = _spike_arg(spike, dev)
  tr = as_tensor(trace, dev, dtype=torch.float32)
  lo, hi = _bounds(w_min, w_max)
  ws = _stdp_workspace(rows, dev)
  st = call(w, out, sp, et, tr, lo, hi, ws, _lib.stream_handle(dev))
  _lib.check(st, name)
  return out


def csr_on_pre_update(w, indices, indptr, spike, trace, w_min=None, w_max=None, *, out=None):
  """brainpy/_src/dnn/linear.py:666-671: a new weight array where every synapse k of a
  spiking pre-synaptic row becomes clip(w[k] + trace[post(k)], w_min, w_max).  ``out=w``
  updates in place."""
  dev = w.device if isinstance(w, torch.Tensor) and w.is_cuda else default_device()
  ind = as_tensor(indices, dev)
  ptr = as_tensor(indptr, dev)
  it = index_type(ind, "indices")
  if index_type(ptr, "indptr") != it:
    raise ValueError("indices and indptr must have the same integer type.")
  m = ptr.shape[0] - 1
  n = int(trace.shape[0])
  if spike.shape[0] != m:
    raise ValueError(f"spike has {spike.shape[0]} entries, the CSR has {m} rows")
  return _plastic("csr_on_pre_update", w, out, spike, trace, w_min, w_max, m,
                  lambda w_, o, sp, et, tr, lo, hi, ws, s: _lib.lib().bp_csr_on_pre_update(
                      _lib.ptr(w_), _lib.ptr(o), _lib.ptr(ind), _lib.ptr(ptr), it, ind.shape[0], m, n, _lib.ptr(sp),
                      et, _lib.ptr(tr), lo, hi, _lib.ptr(ws), ws.numel(), s))


def csc_on_post_update(w, post_ids, indptr, w_ids, spike, trace, w_min=None, w_max=None, *, out=None):
  """brainpy/_src/dnn/linear.py:691-696: a new weight array where, for every spiking
  post-synaptic column, each of its synapses w_ids[k] becomes clip(w + trace[post_ids[k]]);
  (post_ids, indptr, w_ids) is the CSC form from ``connect.csr2csc`` (post_ids hold the
  pre-synaptic ids, as in the reference).  ``out=w`` updates in place."""
  dev = w.device if isinstance(w, torch.Tensor) and w.is_cuda else default_device()
  pid = as_tensor(post_ids, dev)
  ptr = as_tensor(indptr, dev)
  wid = as_tensor(w_ids, dev)
  it = index_type(pid, "post_ids")
  if index_type(ptr, "indptr") != it or index_type(wid, "w_ids") != it:
    raise ValueError("post_ids, indptr and w_ids must have the same integer type.")
  n = ptr.shape[0] - 1
  m = int(trace.shape[0])
  if spike.shape[0] != n:
    raise ValueError(f"spike has {spike.shape[0]} entries, the CSC has {n} columns")
  return _plastic("csc_on_post_update", w, out, spike, trace, w_min, w_max, n,
                  lambda w_, o, sp, et, tr, lo, hi, ws, s: _lib.lib().bp_csc_on_post_update(
                      _lib.ptr(w_), _lib.ptr(o), _lib.ptr(pid), _lib.ptr(ptr), _lib.ptr(wid), it, pid.shape[0], n, m,
                      _lib.ptr(sp), et, _lib.ptr(tr), lo, hi, _lib.ptr(ws), ws.numel(), s))


class _CSRLayer:
  """A fixed CSR connection with a scalar or per-synapse weight (linear.py:490-527)."""

  def __init__(self, conn, weight, transpose: bool = True, shape=None, name: Optional[str] = None):
    if hasattr(conn, "require"):
      indices, indptr = conn.require("csr")
      pre_num, post_num = int(conn.pre_num), int(conn.post_num)
    else:
      indices, indptr = conn
      if shape is None:
        raise ValueError("shape=(pre_num, post_num) is required when the connection is given as (indices, indptr)")
      pre_num, post_num = int(shape[0]), int(shape[1])
    dev = default_device()
    self.indices = as_tensor(indices, dev)
    self.indptr = as_tensor(indptr, dev)
    if self.indptr.numel() != pre_num + 1:
      raise ValueError(f"indptr should have {pre_num + 1} entries, got {self.indptr.numel()}")
    self.pre_num, self.post_num = pre_num, post_num
    self.transpose = bool(transpose)
    if isinstance(weight, (float, int)) and not isinstance(weight, bool):
      self.weight = float(weight)
    else:
      w = as_tensor(np.asarray(weight, np.float32) if not isinstance(weight, torch.Tensor) else weight, dev)
      if w.numel() not in (1, self.indices.numel()):
        raise ValueError(f"weight should be a scalar or have {self.indices.numel()} entries, got {w.numel()}")
      self.weight = w.reshape(-1).to(torch.float32)
    self.name = name

  def __call__(self, x):
    return self.update(x)

  def stdp_update(self, on_pre=None, on_post=None, w_min=None, w_max=None):
    """brainpy/_src/dnn/linear.py:517-543: weight updates on pre-synaptic spikes
    (``on_pre={'spike', 'trace'}``, trace over the post population) and on post-synaptic
    spikes (``on_post``, trace over the pre population).  The weight is updated in place and
    only on the spiking rows/columns; the CSC form is built once, on first use."""
    if not isinstance(self.weight, torch.Tensor):
      raise ValueError("When using STDP to update synaptic weights, the weight cannot be a scalar.")
    if tuple(self.weight.shape) != tuple(self.indices.shape):
      raise ValueError(f"The shape of weight should be the same as the shape of sparse weight "
                       f"{tuple(self.weight.shape)}.")
    with torch.no_grad():
      w = self.weight
      if on_pre is not None:
        csr_on_pre_update(w, self.indices, self.indptr, on_pre["spike"], on_pre["trace"], w_min, w_max, out=w)
      if on_post is not None:
        if not hasattr(self, "_csc"):
          from .connect import csr2csc
          self._csc = csr2csc(self.indices, self.indptr, self.post_num)
        pre_ids, c_indptr, w_ids = self._csc
        csc_on_post_update(w, pre_ids, c_indptr, w_ids, on_post["spike"], on_post["trace"], w_min, w_max, out=w)


class CSRLinear(_CSRLayer):
  """y = x @ W (transpose=True) or W @ x with W a CSR matrix; sparse.csrmv (linear.py:555-609)."""

  def __init__(self, conn, weight, method: str = "cusparse", transpose: bool = True, shape=None,
               name: Optional[str] = None):
    super().__init__(conn, weight, transpose=transpose, shape=shape, name=name)
    self.method = method

  def update(self, x):
    x = as_tensor(x, default_device())
    shape = (self.pre_num, self.post_num)
    return _batched(lambda v: _sparse.csrmv(self.weight, self.indices, self.indptr, v, shape=shape,
                                            transpose=self.transpose, method=self.method), x,
                    lambda b: _sparse.csrmv_batch(self.weight, self.indices, self.indptr, b, shape=shape,
                                                  transpose=self.transpose))


class EventCSRLinear(_CSRLayer):
  """Event-driven y = spikes @ W on a CSR matrix; event.csrmv (linear.py:600-649)."""

  def update(self, x):
    x = as_tensor(x, default_device())
    shape = (self.pre_num, self.post_num)
    return _batched(lambda v: _event.csrmv(self.weight, self.indices, self.indptr, v, shape=shape,
                                           transpose=self.transpose), x,
                    lambda b: _event.csrmv_batch(self.weight, self.indices, self.indptr, b, shape=shape,
                                                 transpose=self.transpose))


class _JitLayer:
  """A just-in-time connection of probability `prob` between num_in inputs and num_out outputs
  (linear.py:805-1280): the seed is drawn once when not given."""

  def __init__(self, num_in: int, num_out: int, prob: float, seed: Optional[int] = None, transpose: bool = False,
               atomic: bool = False, name: Optional[str] = None):
    self.num_in, self.num_out = int(num_in), int(num_out)
    self.prob = float(prob)
    self.seed = int(np.random.randint(0, 1000000)) if seed is None else int(seed)
    self.transpose = bool(transpose)
    self.atomic = bool(atomic)
    self.name = name

  def _call(self, op, x, *weights):
    x = as_tensor(x, default_device())
    return _batched(lambda v: op(v, *weights, self.prob, self.seed, shape=(self.num_out, self.num_in),
                                 transpose=self.transpose, outdim_parallel=not self.atomic), x)

  def __call__(self, x):
    return self.update(x)


class JitFPHomoLinear(_JitLayer):
  """y = M x, M ~ Bernoulli(prob) with one weight; jitconn.mv_prob_homo."""

  def __init__(self, num_in, num_out, prob, weight, seed=None, transpose=False, atomic=False, name=None):
    super().__init__(num_in, num_out, prob, seed, transpose, atomic, name)
    self.weight = float(weight)

  def update(self, x):
    return self._call(_jitconn.mv_prob_homo, x, self.weight)


class JitFPUniformLinear(_JitLayer):
  """y = M x, M ~ Bernoulli(prob) with U[w_low, w_high] weights; jitconn.mv_prob_uniform."""

  def __init__(self, num_in, num_out, prob, w_low, w_high, seed=None, transpose=False, atomic=False, name=None):
    super().__init__(num_in, num_out, prob, seed, transpose, atomic, name)
    self.w_low, self.w_high = float(w_low), float(w_high)

  def update(self, x):
    return self._call(_jitconn.mv_prob_uniform, x, self.w_low, self.w_high)


class JitFPNormalLinear(_JitLayer):
  """y = M x, M ~ Bernoulli(prob) with N(w_mu, w_sigma) weights; jitconn.mv_prob_normal."""

  def __init__(self, num_in, num_out, prob, w_mu, w_sigma, seed=None, transpose=False, atomic=False, name=None):
    super().__init__(num_in, num_out, prob, seed, transpose, atomic, name)
    self.w_mu, self.w_sigma = float(w_mu), float(w_sigma)

  def update(self, x):
    return self._call(_jitconn.mv_prob_normal, x, self.w_mu, self.w_sigma)


class EventJitFPHomoLinear(JitFPHomoLinear):
  """Event-driven JitFPHomoLinear; jitconn.event_mv_prob_homo (linear.py:1044-1120)."""

  def update(self, x):
    return self._call(_jitconn.event_mv_prob_homo, x, self.weight)


class EventJitFPUniformLinear(JitFPUniformLinear):
  """Event-driven JitFPUniformLinear; jitconn.event_mv_prob_uniform (linear.py:1123-1200)."""

  def update(self, x):
    return self._call(_jitconn.event_mv_prob_uniform, x, self.w_low, self.w_high)


class EventJitFPNormalLinear(JitFPNormalLinear):
  """Event-driven JitFPNormalLinear; jitconn.event_mv_prob_normal (linear.py:1203-1280)."""

  def update(self, x):
    return self._call(_jitconn.event_mv_prob_normal, x, self.w_mu, self.w_sigma)
