"""Argument handling shared by the operator front-ends."""
import numpy as np
import torch

from .. import _lib


def default_device():
  if not torch.cuda.is_available():
    raise RuntimeError("brainpy_gb300 operators need a CUDA device (sm_103a); none is available")
  return torch.device("cuda", torch.cuda.current_device())


def as_tensor(x, device=None, dtype=None):
  """Returns `x` as a tensor on the CUDA device (host arrays are copied)."""
  if (dtype is None and isinstance(x, torch.Tensor) and x.is_cuda and device is not None
      and x.device.index == device.index and x.is_contiguous()):
    return x  # already a contiguous tensor on the device
  if device is None:
    device = default_device()
  if isinstance(x, torch.Tensor):
    t = x
  elif isinstance(x, np.ndarray):
    t = torch.from_numpy(np.ascontiguousarray(x))
  else:
    t = torch.as_tensor(x)
  if dtype is not None and t.dtype != dtype:
    t = t.to(dtype)
  if t.device != device:
    t = t.to(device, non_blocking=True)
  return t.contiguous()


_SCALARS = {}


def float_data(data, device):
  """`data` as a 1-D float32 tensor (BrainPy's jnp.atleast_1d(data)).  Python scalars are
  kept as one cached device tensor per (device, value), so a call with a scalar weight does
  not copy it to the device every time."""
  if isinstance(data, (float, int)) and not isinstance(data, bool):
    key = (device, float(data))
    t = _SCALARS.get(key)
    if t is None:
      if len(_SCALARS) >= 256:
        _SCALARS.clear()
      t = torch.tensor([float(data)], dtype=torch.float32, device=device)
      _SCALARS[key] = t
    return t
  t = as_tensor(data, device)
  if t.ndim == 0:
    t = t.reshape(1)
  if t.dtype != torch.float32:
    if t.dtype in (torch.float16, torch.bfloat16, torch.float64):
      raise TypeError(f"only float32 data is supported by this library, got {t.dtype}")
    raise TypeError(f"data must be a float array, got {t.dtype}")
  return t


def index_type(t, what):
  if t.dtype == torch.int32:
    return _lib.BP_I32
  if t.dtype == torch.int64:
    return _lib.BP_I64
  raise ValueError(f"{what} should be a 1D vector with int32 or int64 type.")


def event_type(t, float_rule):
  """bool -> BP_EV_BOOL; float32 -> the given float rule."""
  if t.dtype == torch.bool:
    return _lib.BP_EV_BOOL, t.view(torch.uint8)
  if t.dtype == torch.float32:
    return float_rule, t
  if t.dtype in (torch.float16, torch.bfloat16, torch.float64):
    raise TypeError(f"events of dtype {t.dtype} are not supported by this library (bool or float32)")
  raise TypeError(f"events must be bool or float, got {t.dtype}")
