"""brainpy.math.event on GB300: csrmv, csrmv_taichi, info.

Signatures, argument checks and error types follow
brainpy/_src/math/event/_csr_matvec.py:38-110 (csrmv),
brainpy/_src/math/event/_csr_matvec_taichi.py:344-452 (csrmv_taichi) and
brainpy/_src/math/event/_info_collection.py:24-43 (info).
"""
from typing import Tuple, Union

import torch

from .. import _lib
from ._utils import as_tensor, default_device, event_type, float_data, index_type

__all__ = ["csrmv", "csrmv_taichi", "info"]


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


def _event_csrmv(data, indices, indptr, events, shape, transpose, float_rule, out=None):
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
  """
  return _event_csrmv(data, indices, indptr, events, shape, transpose, _lib.BP_EV_F32_POS)


def csrmv_taichi(data, indices, indptr, events, *, shape, transpose=False):
  """``brainpy.math.event.csrmv_taichi``: as :func:`csrmv`, float events count when ``!= 0``."""
  return _event_csrmv(data, indices, indptr, events, shape, transpose, _lib.BP_EV_F32_NZ)


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
