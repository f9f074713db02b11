"""brainpy.math.sparse on GB300: csrmv, csrmv_taichi, csr_to_dense, csr_to_coo, coo_to_csr.

Signatures and checks follow brainpy/_src/math/sparse/_csr_mv.py:29-123 (csrmv),
brainpy/_src/math/sparse/_csr_mv_taichi.py:160-287 (csrmv_taichi) and
brainpy/_src/math/sparse/_utils.py:20-114 (format conversions).
"""
from typing import Tuple

import torch

from .. import _lib
from . import _grad
from . import event as _event
from ._utils import as_tensor, default_device, float_data, index_type

__all__ = ["csrmv", "csrmv_taichi", "csrmv_batch", "csr_to_dense", "csr_to_coo", "coo_to_csr"]

_METHODS = ("cusparse", "scalar", "vector", "adaptive")


_SPARSE_N_PLAN_MIN_ROW = 256


def _csrmv(data, indices, indptr, vector, shape, transpose, out=None, use_plan=True):
  dev = vector.device if isinstance(vector, torch.Tensor) and vector.is_cuda else default_device()
  data = float_data(data, dev)
  indices = as_tensor(indices, dev)
  indptr = as_tensor(indptr, dev)
  vector = as_tensor(vector, dev)
  if vector.dtype == torch.bool:  # _csr_mv.py:80-81
    vector = vector.to(torch.float32)
  if vector.dtype != torch.float32:
    raise TypeError(f"The types of data and vector should be the same. But we got {data.dtype} != {vector.dtype}.")
  if data.ndim != 1 or indices.ndim != 1 or indptr.ndim != 1 or vector.ndim != 1:
    raise ValueError("data, indices, indptr and vector should be 1D arrays.")
  if data.shape[0] not in (1, indices.shape[0]):
    raise ValueError("The size of data should be 1 or be consistent with indices.")
  if len(shape) != 2:
    raise ValueError("shape should be a length-2 tuple.")
  m, n = int(shape[0]), int(shape[1])
  if indptr.shape[0] != m + 1:
    raise ValueError(f"indptr should have shape ({m + 1},), got {tuple(indptr.shape)}.")
  if vector.shape[0] != (m if transpose else n):
    raise ValueError(f"Shape mismatch, vec ({vector.shape[0]},) and mat {tuple(shape)} with transpose={transpose}.")
  itype = index_type(indices, "indices")
  if index_type(indptr, "indptr") != itype:
    raise ValueError("indices and indptr must have the same integer type.")
  # y = A x gathers the vector: from a shared-memory tile of it on the plan, from L2 in the
  # plain row kernel.  Rows shorter than _SPARSE_N_PLAN_MIN_ROW entries on average leave too
  # few entries per (row, tile) segment for the plan to pay (N = 1e6: 1.03 ms on the plan
  # against 0.40 ms plain at fan-out 100; 1.71 against 3.36 ms at fan-out 1000).
  if use_plan and (transpose or indices.shape[0] >= _SPARSE_N_PLAN_MIN_ROW * max(m, 1)):
    plan = _event._cached_plan(data, indices, indptr, (m, n), routed=False)
    if plan is not None:
      if transpose:
        return plan.sparse_t(vector, None if plan.heter else data, out=out)
      return plan.sparse_n(vector, None if plan.heter else data, out=out)
  n_out = n if transpose else m
  if out is None:
    out = torch.empty(n_out, dtype=torch.float32, device=dev)
  L = _lib.lib()
  st = L.bp_csrmv(_lib.ptr(data), data.shape[0], _lib.ptr(indices), _lib.ptr(indptr), itype, indices.shape[0],
                  _lib.ptr(vector), m, n, int(bool(transpose)), _lib.ptr(out), _lib.stream_handle(dev))
  _lib.check(st, "sparse.csrmv")
  return out


def csrmv(data, indices, indptr, vector, *, shape: Tuple[int, int], transpose: bool = False,
          method: str = "cusparse") -> torch.Tensor:
  """Product of a CSR matrix and a dense vector (``brainpy.math.sparse.csrmv``).

  Every ``method`` of the reference ("cusparse", "scalar", "vector", "adaptive") runs the
  same sm_103a kernels here; an unknown method raises ValueError as in the reference."""
  if method not in _METHODS:
    raise ValueError(f"Only support methods: cusparse, scalar, vector, and adaptive. But we got {method}.")
  return _dispatch(data, indices, indptr, vector, shape, bool(transpose))


def csrmv_taichi(data, indices, indptr, vector, *, shape: Tuple[int, int], transpose: bool = False):
  """``brainpy.math.sparse.csrmv_taichi``."""
  return _dispatch(data, indices, indptr, vector, shape, bool(transpose))


def _dispatch(data, indices, indptr, vector, shape, transpose):
  """The kernels directly, or -- when data or vector needs a gradient -- through the
  reference's differentiation rules (brainpy/_src/math/sparse/_csr_mv.py:211-240)."""
  if _grad.wanted(data, vector):
    dev = vector.device if isinstance(vector, torch.Tensor) and vector.is_cuda else default_device()
    d = float_data(data, dev)
    v = as_tensor(vector, dev)
    if v.dtype == torch.bool:
      v = v.to(torch.float32)
    return _grad.SparseCSRMV.apply(d, v, as_tensor(indices, dev), as_tensor(indptr, dev),
                                   (int(shape[0]), int(shape[1])), transpose)
  return _csrmv(data, indices, indptr, vector, shape, transpose)


def csrmv_batch(data, indices, indptr, vectors, *, shape: Tuple[int, int], transpose: bool = False):
  """csrmv mapped over the leading axis of a (B, len) batch of dense vectors: (B, out).  A
  transpose product on a planned matrix runs the batch in one launch pair
  (bp_csrmv_planned_batch); other cases run the single-vector kernels row by row (the
  reference's batching rule is a sequential scan, brainpy/_src/math/op_register/utils.py:16-38)."""
  dev = vectors.device if isinstance(vectors, torch.Tensor) and vectors.is_cuda else default_device()
  vectors = as_tensor(vectors, dev)
  if vectors.ndim != 2:
    raise ValueError(f"vectors should be a 2D (batch, length) array, got {vectors.ndim}-D.")
  if vectors.dtype == torch.bool:
    vectors = vectors.to(torch.float32)
  m, n = int(shape[0]), int(shape[1])
  if _grad.wanted(data, vectors):
    rows = [_dispatch(data, indices, indptr, vectors[b], shape, bool(transpose)) for b in range(vectors.shape[0])]
    return torch.stack(rows) if rows else torch.empty((0, n if transpose else m), device=dev)
  d = float_data(data, dev)
  indices = as_tensor(indices, dev)
  indptr = as_tensor(indptr, dev)
  if transpose and vectors.shape[0] > 0:
    if indptr.shape[0] != m + 1:
      raise ValueError(f"indptr should have shape ({m + 1},), got {tuple(indptr.shape)}.")
    if vectors.shape[1] != m:
      raise ValueError(f"Shape mismatch, vec ({vectors.shape[1]},) and mat {tuple(shape)} with transpose=True.")
    if d.shape[0] not in (1, indices.shape[0]):
      raise ValueError("The size of data should be 1 or be consistent with indices.")
    plan = _event._cached_plan(d, indices, indptr, (m, n), routed=False)
    if plan is not None:
      return plan.sparse_t_batch(vectors, None if plan.heter else d)
  out = torch.empty((vectors.shape[0], n if transpose else m), dtype=torch.float32, device=dev)
  for b in range(vectors.shape[0]):
    _csrmv(d, indices, indptr, vectors[b], shape, bool(transpose), out=out[b])
  return out


def csr_to_coo(indices, indptr):
  """(row, col) of every stored entry, row ids in indptr's dtype."""
  dev = indices.device if isinstance(indices, torch.Tensor) and indices.is_cuda else default_device()
  indices = as_tensor(indices, dev)
  indptr = as_tensor(indptr, dev)
  itype = index_type(indptr, "indptr")
  rows = torch.empty(indices.shape[0], dtype=indptr.dtype, device=dev)
  st = _lib.lib().bp_csr_to_coo(_lib.ptr(indptr), itype, indptr.shape[0] - 1, indices.shape[0], _lib.ptr(rows),
                                _lib.stream_handle(dev))
  _lib.check(st, "sparse.csr_to_coo")
  return rows, indices


def csr_to_dense(data, indices, indptr, *, shape: Tuple[int, int]):
  """Dense (shape) matrix of a CSR matrix; duplicate entries add up."""
  dev = indices.device if isinstance(indices, torch.Tensor) and indices.is_cuda else default_device()
  data = float_data(data, dev)
  indices = as_tensor(indices, dev)
  indptr = as_tensor(indptr, dev)
  itype = index_type(indices, "indices")
  m, n = int(shape[0]), int(shape[1])
  if indptr.shape[0] != m + 1:
    raise ValueError(f"indptr should have shape ({m + 1},).")
  dense = torch.empty((m, n), dtype=torch.float32, device=dev)
  st = _lib.lib().bp_csr_to_dense(_lib.ptr(data), data.shape[0], _lib.ptr(indices), _lib.ptr(indptr), itype,
                                  indices.shape[0], m, n, _lib.ptr(dense), _lib.stream_handle(dev))
  _lib.check(st, "sparse.csr_to_dense")
  return dense


def coo_to_csr(pre_ids, post_ids, *, num_row: int):
  """(indices, indptr) of a COO connection list (stable sort by pre id), as
  brainpy/_src/math/sparse/_utils.py:20-41.  A one-time setup conversion built from torch's
  stable sort and cumulative sum."""
  dev = pre_ids.device if isinstance(pre_ids, torch.Tensor) and pre_ids.is_cuda else default_device()
  pre = as_tensor(pre_ids, dev).to(torch.int64)
  post = as_tensor(post_ids, dev)
  order = torch.sort(pre, stable=True).indices
  indices = post[order]
  counts = torch.bincount(pre, minlength=int(num_row))[: int(num_row)]
  indptr = torch.zeros(int(num_row) + 1, dtype=post.dtype, device=dev)
  indptr[1:] = torch.cumsum(counts, 0).to(post.dtype)
  return indices, indptr
