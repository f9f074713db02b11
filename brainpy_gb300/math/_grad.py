"""Reverse- and forward-mode rules of the propagation operators (torch.autograd.Function).

The rules are the reference's JVP and transpose definitions:
* event.csrmv -- brainpy/_src/math/event/_csr_matvec.py:521-551: tangent of the values is
  csrmv(values_dot, events); tangent of the events is sparse.csrmv(values, events_dot) (the
  events enter linearly); cotangent of the events is sparse.csrmv(values, ct, not transpose);
  cotangent of the values is <ct, csrmv(1, events)> for a scalar weight and
  events[row] * ct[col] (transpose) or events[col] * ct[row] per stored entry otherwise.
* sparse.csrmv -- brainpy/_src/math/sparse/_csr_mv.py:211-240: the same with a dense vector.
* jitconn -- brainpy/_src/math/jitconn/_matvec_taichi.py:138-171 (and the uniform/normal
  twins :480-495, :767-782, used by the event operators too): the cotangent of the vector is
  the non-event product of ct with transpose and outdim_parallel both flipped, which
  regenerates the same lane streams and hence the transposed matrix; the scalar weight of the
  homogeneous operators gets <ct, M v / w>.  The reference computes that last one as
  sum(mv(ct, 1, same flags) * v), which only type-checks for square shapes; here it is the
  exact derivative <ct, mv(v, 1, same flags)>.  w_low/w_high and w_mu/w_sigma, as in the
  reference, take no gradient.

The operators route through these Functions only when an input requires a gradient or carries
a forward-mode tangent; otherwise they call the kernels directly.
"""
import torch
from torch.autograd import forward_ad as _fwad

from .. import _lib

__all__ = ["wanted"]


def _has_tangent(x):
  return isinstance(x, torch.Tensor) and _fwad.unpack_dual(x).tangent is not None


def wanted(*xs) -> bool:
  """True when one of the tensors needs a reverse-mode gradient or has a forward tangent."""
  if torch.is_grad_enabled() and any(isinstance(x, torch.Tensor) and x.requires_grad for x in xs):
    return True
  if getattr(_fwad, "_current_level", -1) >= 0:
    return any(_has_tangent(x) for x in xs)
  return False


def sampled_outer(x, y, indices, indptr, m, n):
  """out[j] = x[row(j)] * y[indices[j]] for every stored entry (the CSR weight cotangent)."""
  from ._utils import index_type
  x = x.detach().to(torch.float32).contiguous()
  y = y.detach().to(torch.float32).contiguous()
  out = torch.empty(indices.shape[0], dtype=torch.float32, device=indices.device)
  L = _lib.lib()
  st = L.bp_csr_sampled_outer(_lib.ptr(x), _lib.ptr(y), _lib.ptr(indices), _lib.ptr(indptr),
                              index_type(indices, "indices"), indices.shape[0], m, n, _lib.ptr(out),
                              _lib.stream_handle(indices.device))
  _lib.check(st, "csr_sampled_outer")
  return out


def _data_cotangent(data, ct, vec, indices, indptr, shape, transpose, product):
  """Cotangent of the CSR values: <ct, product(1)> for one weight, the sampled outer product
  otherwise (vec is the events or the dense vector)."""
  m, n = int(shape[0]), int(shape[1])
  if data.numel() == 1:
    ones = torch.ones(1, dtype=torch.float32, device=ct.device)
    return torch.dot(ct, product(ones)).reshape(data.shape)
  v = vec.to(torch.float32)
  return sampled_outer(v, ct, indices, indptr, m, n) if transpose else sampled_outer(ct, v, indices, indptr, m, n)


class EventCSRMV(torch.autograd.Function):
  """event.csrmv / event.csrmv_taichi with the reference's differentiation rules."""

  @staticmethod
  def forward(data, events, indices, indptr, shape, transpose, float_rule):
    from . import event
    return event._event_csrmv(data.detach(), indices, indptr, events.detach(), shape, transpose, float_rule)

  @staticmethod
  def setup_context(ctx, inputs, output):
    data, events, indices, indptr, shape, transpose, float_rule = inputs
    ctx.save_for_backward(data, events, indices, indptr)
    ctx.save_for_forward(data, events, indices, indptr)
    ctx.shape, ctx.transpose, ctx.float_rule = shape, bool(transpose), float_rule
    ctx.set_materialize_grads(False)

  @staticmethod
  def backward(ctx, ct):
    if ct is None:
      return (None,) * 7
    from . import event, sparse
    data, events, indices, indptr = ctx.saved_tensors
    ct = ct.contiguous()
    g_data = g_events = None
    if ctx.needs_input_grad[0]:
      g_data = _data_cotangent(
          data, ct, events, indices, indptr, ctx.shape, ctx.transpose,
          lambda w: event._event_csrmv(w, indices, indptr, events.detach(), ctx.shape, ctx.transpose, ctx.float_rule))
    if ctx.needs_input_grad[1]:
      g_events = sparse._csrmv(data.detach(), indices, indptr, ct, ctx.shape, not ctx.transpose)
    return g_data, g_events, None, None, None, None, None

  @staticmethod
  def jvp(ctx, d_data, d_events, *_):
    from . import event, sparse
    data, events, indices, indptr = ctx.saved_tensors
    out = None
    if d_data is not None:
      out = event._event_csrmv(d_data.contiguous(), indices, indptr, events, ctx.shape, ctx.transpose,
                               ctx.float_rule, use_plan=False)
    if d_events is not None:
      d = sparse._csrmv(data, indices, indptr, d_events.contiguous(), ctx.shape, ctx.transpose, use_plan=False)
      out = d if out is None else out + d
    return out


class SparseCSRMV(torch.autograd.Function):
  """sparse.csrmv / sparse.csrmv_taichi with the reference's differentiation rules."""

  @staticmethod
  def forward(data, vector, indices, indptr, shape, transpose):
    from . import sparse
    return sparse._csrmv(data.detach(), indices, indptr, vector.detach(), shape, transpose)

  @staticmethod
  def setup_context(ctx, inputs, output):
    data, vector, indices, indptr, shape, transpose = inputs
    ctx.save_for_backward(data, vector, indices, indptr)
    ctx.save_for_forward(data, vector, indices, indptr)
    ctx.shape, ctx.transpose = shape, bool(transpose)
    ctx.set_materialize_grads(False)

  @staticmethod
  def backward(ctx, ct):
    if ct is None:
      return (None,) * 6
    from . import sparse
    data, vector, indices, indptr = ctx.saved_tensors
    ct = ct.contiguous()
    g_data = g_vec = None
    if ctx.needs_input_grad[0]:
      g_data = _data_cotangent(
          data, ct, vector, indices, indptr, ctx.shape, ctx.transpose,
          lambda w: sparse._csrmv(w, indices, indptr, vector.detach(), ctx.shape, ctx.transpose))
    if ctx.needs_input_grad[1]:
      g_vec = sparse._csrmv(data.detach(), indices, indptr, ct, ctx.shape, not ctx.transpose)
    return g_data, g_vec, None, None, None, None

  @staticmethod
  def jvp(ctx, d_data, d_vec, *_):
    from . import sparse
    data, vector, indices, indptr = ctx.saved_tensors
    out = None
    if d_data is not None:
      out = sparse._csrmv(d_data.contiguous(), indices, indptr, vector, ctx.shape, ctx.transpose, use_plan=False)
    if d_vec is not None:
      d = sparse._csrmv(data, indices, indptr, d_vec.contiguous(), ctx.shape, ctx.transpose, use_plan=False)
      out = d if out is None else out + d
    return out


class JitMV(torch.autograd.Function):
  """The jitconn operators (event and non-event, homo/uniform/normal) with the reference's
  differentiation rules.  `weight` is the homogeneous weight as a tensor (None for the other
  kinds, whose p0/p1 are plain numbers); `seed` is already resolved."""

  @staticmethod
  def forward(vector, weight, kind, event, p0, p1, conn_prob, seed, shape, transpose, outdim_parallel, taichi,
              variant):
    from . import jitconn
    w0 = float(weight.detach().reshape(-1)[0]) if weight is not None else p0
    return jitconn._mv(kind, event, vector.detach(), w0, p1, conn_prob, seed, shape, transpose, outdim_parallel,
                       taichi, variant)

  @staticmethod
  def setup_context(ctx, inputs, output):
    (vector, weight, kind, event, p0, p1, conn_prob, seed, shape, transpose, outdim_parallel, taichi,
     variant) = inputs
    ctx.save_for_backward(vector)
    ctx.save_for_forward(vector)
    ctx.w0 = float(weight.detach().reshape(-1)[0]) if weight is not None else p0
    ctx.w_shape = weight.shape if weight is not None else None
    ctx.args = (kind, event, p1, conn_prob, seed, shape, bool(transpose), bool(outdim_parallel), taichi, variant)
    ctx.set_materialize_grads(False)

  @staticmethod
  def backward(ctx, ct):
    if ct is None:
      return (None,) * 13
    from . import jitconn
    (vector,) = ctx.saved_tensors
    kind, event, p1, conn_prob, seed, shape, transpose, outdim_parallel, taichi, variant = ctx.args
    ct = ct.contiguous()
    g_vec = g_w = None
    if ctx.needs_input_grad[0]:
      g_vec = jitconn._mv(kind, False, ct, ctx.w0, p1, conn_prob, seed, shape, not transpose, not outdim_parallel,
                          taichi, variant)
    if ctx.needs_input_grad[1]:
      unit = jitconn._mv(kind, event, vector.detach(), 1.0, p1, conn_prob, seed, shape, transpose, outdim_parallel,
                         taichi, variant)
      g_w = torch.dot(ct, unit).reshape(ctx.w_shape)
    return (g_vec, g_w) + (None,) * 11

  @staticmethod
  def jvp(ctx, d_vec, d_w, *_):
    from . import jitconn
    (vector,) = ctx.saved_tensors
    kind, event, p1, conn_prob, seed, shape, transpose, outdim_parallel, taichi, variant = ctx.args
    out = None
    if d_vec is not None:
      out = jitconn._mv(kind, False, d_vec.contiguous(), ctx.w0, p1, conn_prob, seed, shape, transpose,
                        outdim_parallel, taichi, variant)
    if d_w is not None:
      unit = jitconn._mv(kind, event, vector, 1.0, p1, conn_prob, seed, shape, transpose, outdim_parallel, taichi,
                         variant)
      d = unit * d_w.reshape(-1)[0]
      out = d if out is None else out + d
    return out
