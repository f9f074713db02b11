"""brainpy.math.jitconn on GB300.

Signatures and checks follow brainpy/_src/math/jitconn/_event_matvec.py:32-123 (public
event ops), _matvec.py:27-260 (public mv ops) and the *_taichi twins
(_event_matvec_taichi.py:340-408 and siblings, _matvec_taichi.py:174-318).

The connectivity is the reference's Taichi GPU algorithm (32 LFSR88 lane streams per
output row for outdim_parallel=True, per input column otherwise), regenerated on every
call by libbpgpu; ``variant="cpu"`` selects the reference's Taichi CPU algorithm, which
generates a different matrix.
"""
import math
from typing import Optional, Tuple

import numpy as np
import torch

from .. import _lib
from . import _grad
from ._utils import as_tensor, default_device

__all__ = [
    "event_mv_prob_homo", "event_mv_prob_uniform", "event_mv_prob_normal",
    "mv_prob_homo", "mv_prob_uniform", "mv_prob_normal",
    "event_mv_prob_homo_taichi", "event_mv_prob_uniform_taichi", "event_mv_prob_normal_taichi",
    "mv_prob_homo_taichi", "mv_prob_uniform_taichi", "mv_prob_normal_taichi",
    "get_conn_matrix", "conn_len",
]

_KIND = {"homo": _lib.BP_JC_HOMO, "uniform": _lib.BP_JC_UNIFORM, "normal": _lib.BP_JC_NORMAL}
_VARIANT = {"gpu": _lib.BP_JC_TAICHI_GPU, "cpu": _lib.BP_JC_TAICHI_CPU}


def conn_len(conn_prob, taichi=False) -> int:
  """int32(ceil(1 / conn_prob) * 2 - 1).

  Public ops compute 1/conn_prob in float32 (_event_matvec.py:44-45); the *_taichi ops
  in Python double before jnp.ceil turns it into float32 (_event_matvec_taichi.py:401-402)."""
  if taichi:
    q = np.float32(1.0 / float(conn_prob))
  else:
    q = np.float32(1.0) / np.float32(conn_prob)
  return int(np.float32(math.ceil(q)) * np.float32(2) - np.float32(1))


def _seed(seed, taichi):
  if seed is None:
    seed = int(np.random.randint(0, int(1e8)))
  return int(seed) & 0xFFFFFFFF


def _scalar(x, name):
  if isinstance(x, torch.Tensor):
    if x.numel() != 1:
      raise ValueError(f"{name} must be a 1D scalar.")
    return float(x.reshape(-1)[0].item())
  if isinstance(x, np.ndarray):
    if x.size != 1:
      raise ValueError(f"{name} must be a 1D scalar.")
    return float(x.reshape(-1)[0])
  return float(x)


def _general_checking(vec, shape, outdim_parallel, transpose):
  """brainpy/_src/math/jitconn/_matvec_taichi.py:174-207: returns (num_row, num_col)."""
  if vec.ndim != 1:
    raise ValueError("vector should be a 1D vector.")
  if len(shape) != 2:
    raise ValueError("shape should be a length-2 tuple.")
  if not isinstance(outdim_parallel, bool):
    raise ValueError("outdim_parallel must be boolean value.")
  if not isinstance(transpose, bool):
    raise ValueError("transpose must be boolean value.")
  if transpose:
    if vec.shape[0] != shape[0]:
      raise ValueError(f"Shape mismatch, vec {tuple(vec.shape)} @ mat {tuple(shape)}.")
    return int(shape[1]), int(shape[0])
  if vec.shape[0] != shape[1]:
    raise ValueError(f"Shape mismatch, mat {tuple(shape)} @ vec ({vec.shape[0]},).")
  return int(shape[0]), int(shape[1])


def _mv(kind, event, vec, p0, p1, conn_prob, seed, shape, transpose, outdim_parallel, taichi, variant="gpu",
        out=None):
  dev = vec.device if isinstance(vec, torch.Tensor) and vec.is_cuda else default_device()
  vec = as_tensor(vec, dev)
  num_row, num_col = _general_checking(vec, shape, outdim_parallel, transpose)
  if event:
    if vec.dtype == torch.bool:
      vk, v = _lib.BP_VEC_EVENT_BOOL, vec.view(torch.uint8)
    elif vec.dtype == torch.float32:
      vk, v = _lib.BP_VEC_EVENT_F32, vec
    else:
      raise TypeError(f"events must be bool or float32, got {vec.dtype}")
  else:
    if vec.dtype == torch.bool:
      vec = vec.to(torch.float32)
    if vec.dtype != torch.float32:
      raise TypeError(f"vector must be float32, got {vec.dtype}")
    vk, v = _lib.BP_VEC_DENSE_F32, vec
  clen = conn_len(conn_prob, taichi)
  s = _seed(seed, taichi)
  if out is None:
    out = torch.empty(num_row, dtype=torch.float32, device=dev)
  L = _lib.lib()
  st = L.bp_jitconn_mv(_KIND[kind], vk, _lib.ptr(v), num_col, num_row, float(p0), float(p1), clen, s,
                       int(outdim_parallel), _VARIANT[variant], _lib.ptr(out), _lib.stream_handle(dev))
  _lib.check(st, f"jitconn.{'event_' if event else ''}mv_prob_{kind}")
  return out


def _doc(kind, event):
  w = {"homo": "weight", "uniform": "w_low, w_high", "normal": "w_mu, w_sigma"}[kind]
  return (f"y = M @ v with M ~ Bernoulli(conn_prob) generated just in time ({w}); same arguments as "
          f"brainpy.math.jitconn.{'event_' if event else ''}mv_prob_{kind}.")


def _grad_mv(kind, event, vector, weight, p0, p1, conn_prob, seed, shape, transpose, outdim_parallel, taichi,
             variant):
  """The operator through the reference's differentiation rules (a fixed seed is drawn first,
  so that the backward pass regenerates the same matrix)."""
  dev = vector.device if isinstance(vector, torch.Tensor) and vector.is_cuda else default_device()
  v = as_tensor(vector, dev)
  if not event and v.dtype == torch.bool:
    v = v.to(torch.float32)
  w = None
  if isinstance(weight, torch.Tensor) and _grad.wanted(weight):
    if weight.numel() != 1:
      raise ValueError("weight must be a 1D scalar.")
    w = weight
  elif weight is not None:
    p0 = _scalar(weight, "weight")
  return _grad.JitMV.apply(v, w, kind, event, p0, p1, conn_prob, _seed(seed, taichi), tuple(shape), bool(transpose),
                           bool(outdim_parallel), taichi, variant)


def _make(kind, event, taichi):
  """One public operator with the reference's signature for `kind`."""
  if kind == "homo":
    def op(vector, weight, conn_prob, seed: Optional[int] = None, *, shape: Tuple[int, int],
           transpose: bool = False, outdim_parallel: bool = True, variant: str = "gpu"):
      if _grad.wanted(vector, weight):
        return _grad_mv(kind, event, vector, weight, 0.0, 0.0, conn_prob, seed, shape, transpose, outdim_parallel,
                        taichi, variant)
      return _mv(kind, event, vector, _scalar(weight, "weight"), 0.0, conn_prob, seed, shape, transpose,
                 outdim_parallel, taichi, variant)
  elif kind == "uniform":
    def op(vector, w_low, w_high, conn_prob, seed: Optional[int] = None, *, shape: Tuple[int, int],
           transpose: bool = False, outdim_parallel: bool = True, variant: str = "gpu"):
      if _grad.wanted(vector):
        return _grad_mv(kind, event, vector, None, _scalar(w_low, "w_low"), _scalar(w_high, "w_high"), conn_prob,
                        seed, shape, transpose, outdim_parallel, taichi, variant)
      return _mv(kind, event, vector, _scalar(w_low, "w_low"), _scalar(w_high, "w_high"), conn_prob, seed, shape,
                 transpose, outdim_parallel, taichi, variant)
  else:
    def op(vector, w_mu, w_sigma, conn_prob, seed: Optional[int] = None, *, shape: Tuple[int, int],
           transpose: bool = False, outdim_parallel: bool = True, variant: str = "gpu"):
      if _grad.wanted(vector):
        return _grad_mv(kind, event, vector, None, _scalar(w_mu, "w_mu"), _scalar(w_sigma, "w_sigma"), conn_prob,
                        seed, shape, transpose, outdim_parallel, taichi, variant)
      return _mv(kind, event, vector, _scalar(w_mu, "w_mu"), _scalar(w_sigma, "w_sigma"), conn_prob, seed, shape,
                 transpose, outdim_parallel, taichi, variant)
  op.__name__ = f"{'event_' if event else ''}mv_prob_{kind}{'_taichi' if taichi else ''}"
  op.__doc__ = _doc(kind, event) + (" Taichi twin: conn_len from a double-precision 1/conn_prob." if taichi else "")
  return op


event_mv_prob_homo = _make("homo", True, False)
event_mv_prob_uniform = _make("uniform", True, False)
event_mv_prob_normal = _make("normal", True, False)
mv_prob_homo = _make("homo", False, False)
mv_prob_uniform = _make("uniform", False, False)
mv_prob_normal = _make("normal", False, False)
event_mv_prob_homo_taichi = _make("homo", True, True)
event_mv_prob_uniform_taichi = _make("uniform", True, True)
event_mv_prob_normal_taichi = _make("normal", True, True)
mv_prob_homo_taichi = _make("homo", False, True)
mv_prob_uniform_taichi = _make("uniform", False, True)
mv_prob_normal_taichi = _make("normal", False, True)


def get_conn_matrix(kind, p0, p1, conn_prob, seed, *, shape, transpose=False, outdim_parallel=True, variant="gpu",
                    taichi=False, device=None):
  """The just-in-time matrix written out densely as the kernels see it: (num_row, num_col)
  = (out_len, in_len), i.e. M for transpose=False and M^T (as generated) for transpose=True."""
  dev = device or default_device()
  num_row, num_col = (int(shape[1]), int(shape[0])) if transpose else (int(shape[0]), int(shape[1]))
  dense = torch.empty((num_row, num_col), dtype=torch.float32, device=dev)
  L = _lib.lib()
  st = L.bp_jitconn_dense(_KIND[kind], float(p0), float(p1), conn_len(conn_prob, taichi), _seed(seed, taichi),
                          num_row, num_col, int(outdim_parallel), _VARIANT[variant], _lib.ptr(dense),
                          _lib.stream_handle(dev))
  _lib.check(st, "jitconn.get_conn_matrix")
  return dense
