"""ctypes binding of libbpgpu.so.

The library is the only compute path: if it is missing, importing an operator
module raises immediately (there is no CPU or PyTorch fallback).
"""
import ctypes
import os

import torch

from . import _build

_LIB = None

BP_OK, BP_EINVAL, BP_ESHAPE, BP_EDTYPE, BP_ENOMEM, BP_ETIMEOUT, BP_ECUDA, BP_ENOTSUP = range(8)
BP_I32, BP_I64 = 0, 1
BP_EV_BOOL, BP_EV_F32_POS, BP_EV_F32_NZ = 0, 1, 2
BP_JC_HOMO, BP_JC_UNIFORM, BP_JC_NORMAL = 0, 1, 2
BP_VEC_EVENT_BOOL, BP_VEC_EVENT_F32, BP_VEC_DENSE_F32 = 0, 1, 2
BP_JC_TAICHI_GPU, BP_JC_TAICHI_CPU = 0, 1

_c_i64 = ctypes.c_int64
_c_i32 = ctypes.c_int32
_c_u32 = ctypes.c_uint32
_c_f32 = ctypes.c_float
_c_size = ctypes.c_size_t
_c_ptr = ctypes.c_void_p

# name -> (restype, argtypes); kept in the same order as include/bpgpu.h
SIGNATURES = {
    "bp_status_string": (ctypes.c_char_p, [_c_i32]),
    "bp_last_error": (ctypes.c_char_p, []),
    "bp_version": (_c_i32, []),
    "bp_event_info_workspace_size": (_c_size, [_c_i64]),
    "bp_event_info": (_c_i32, [_c_ptr, _c_i32, _c_i64, _c_ptr, _c_ptr, _c_ptr, _c_size, _c_ptr]),
    "bp_event_csrmv_workspace_size": (_c_size, [_c_i64, _c_i64, _c_i32]),
    "bp_event_csrmv": (_c_i32, [_c_ptr, _c_i64, _c_ptr, _c_ptr, _c_i32, _c_i64, _c_ptr, _c_i32, _c_i64, _c_i64,
                                _c_i32, _c_ptr, _c_ptr, _c_size, _c_ptr]),
    "bp_csrmv": (_c_i32, [_c_ptr, _c_i64, _c_ptr, _c_ptr, _c_i32, _c_i64, _c_ptr, _c_i64, _c_i64, _c_i32, _c_ptr,
                          _c_ptr]),
    "bp_csr_to_coo": (_c_i32, [_c_ptr, _c_i32, _c_i64, _c_i64, _c_ptr, _c_ptr]),
    "bp_fixed_prob_row_lengths": (_c_i32, [_c_i64, _c_i64, _c_i32, ctypes.c_uint64, _c_i32, _c_i32, _c_ptr, _c_ptr,
                                           _c_ptr]),
    "bp_fixed_prob_fill": (_c_i32, [_c_i64, _c_i64, _c_i32, ctypes.c_uint64, _c_i32, _c_i32, _c_ptr, _c_ptr, _c_ptr,
                                    _c_ptr]),
    "bp_stdp_workspace_size": (_c_size, [_c_i64]),
    "bp_spike_ring_record": (_c_i32, [_c_ptr, _c_i64, _c_ptr, _c_i32, _c_i64, _c_ptr, _c_ptr]),
    "bp_spike_ring_read": (_c_i32, [_c_ptr, _c_i32, _c_i64, _c_i64, _c_i64, _c_i32, _c_i64, _c_ptr, _c_ptr, _c_ptr]),
    "bp_csr_on_pre_update": (_c_i32, [_c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_i32, _c_i64, _c_i64, _c_i64, _c_ptr, _c_i32,
                                      _c_ptr, _c_f32, _c_f32, _c_ptr, _c_size, _c_ptr]),
    "bp_csc_on_post_update": (_c_i32, [_c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_i32, _c_i64, _c_i64, _c_i64, _c_ptr,
                                       _c_i32, _c_ptr, _c_f32, _c_f32, _c_ptr, _c_size, _c_ptr]),
    "bp_csr_sampled_outer": (_c_i32, [_c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_i32, _c_i64, _c_i64, _c_i64, _c_ptr,
                                      _c_ptr]),
    "bp_csr_to_dense": (_c_i32, [_c_ptr, _c_i64, _c_ptr, _c_ptr, _c_i32, _c_i64, _c_i64, _c_i64, _c_ptr, _c_ptr]),
    "bp_jitconn_mv": (_c_i32, [_c_i32, _c_i32, _c_ptr, _c_i64, _c_i64, _c_f32, _c_f32, _c_i32, _c_u32, _c_i32, _c_i32,
                               _c_ptr, _c_ptr]),
    "bp_jitconn_csr": (_c_i32, [_c_i32, _c_i32, _c_u32, _c_i64, _c_i64, _c_ptr, _c_ptr, _c_i64, _c_ptr, _c_i64, _c_i32,
                                _c_ptr]),
    "bp_jitconn_dense": (_c_i32, [_c_i32, _c_f32, _c_f32, _c_i32, _c_u32, _c_i64, _c_i64, _c_i32, _c_i32, _c_ptr,
                                  _c_ptr]),
    "bp_csr_plan_default_tile": (_c_i32, [_c_i64, _c_i32]),
    "bp_csr_plan_count_tile": (_c_i32, [_c_i64]),
    "bp_csr_plan_fix_weights": (_c_i32, [_c_ptr, _c_i32, _c_f32, _c_ptr, _c_ptr, _c_ptr, _c_i64, _c_ptr, _c_i32,
                                         _c_ptr]),
    "bp_csr_plan_fix_interleave_bytes": (_c_size, [_c_ptr, _c_i32]),
    "bp_csr_plan_fix_interleave": (_c_i32, [_c_ptr, _c_i32, _c_ptr, _c_size, _c_ptr, _c_ptr]),
    "bp_event_csrmv_planned_fixed": (_c_i32, [_c_ptr, _c_ptr, _c_i32, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_i64,
                                              _c_ptr, _c_i32, _c_ptr, _c_i32, _c_ptr, _c_size, _c_ptr]),
    "bp_csr_plan_variants": (_c_i32, [_c_ptr, _c_i32]),
    "bp_csr_plan_bytes": (_c_size, [_c_i64, _c_i64, _c_i64, _c_i32, _c_i32]),
    "bp_csr_plan_build": (_c_i32, [_c_ptr, _c_i64, _c_ptr, _c_ptr, _c_i32, _c_i64, _c_i64, _c_i64, _c_i32, _c_ptr,
                                   _c_size, _c_ptr, _c_ptr]),
    "bp_event_csrmv_planned_workspace_size": (_c_size, [_c_ptr]),
    "bp_event_csrmv_planned": (_c_i32, [_c_ptr, _c_ptr, _c_ptr, _c_i32, _c_ptr, _c_i32, _c_ptr, _c_size, _c_ptr]),
    "bp_csrmv_planned": (_c_i32, [_c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_i32, _c_ptr, _c_size, _c_ptr]),
    "bp_event_csrmv_planned_batch_workspace_size": (_c_size, [_c_ptr, _c_i32]),
    "bp_csrmv_planned_n_workspace_size": (_c_size, [_c_ptr]),
    "bp_csrmv_planned_n": (_c_i32, [_c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_size, _c_ptr]),
    "bp_event_csrmv_planned_batch": (_c_i32, [_c_ptr, _c_ptr, _c_ptr, _c_i32, _c_i32, _c_ptr, _c_i32, _c_ptr, _c_size,
                                              _c_ptr]),
    "bp_csrmv_planned_batch": (_c_i32, [_c_ptr, _c_ptr, _c_ptr, _c_i32, _c_ptr, _c_i32, _c_ptr, _c_size, _c_ptr]),
    "bp_csr_plan_arrays": (_c_i32, [_c_ptr, ctypes.POINTER(_c_ptr), ctypes.POINTER(_c_ptr), ctypes.POINTER(_c_ptr)]),
    "bp_lif_coba_step": (_c_i32, [_c_ptr, _c_i64, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_i32,
                                  _c_f32, _c_ptr]),
    "bp_lif_coba_step_dev": (_c_i32, [_c_ptr, _c_i64, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr,
                                      _c_i32, _c_f32, _c_ptr]),
    "bp_net_max_tiles": (_c_i32, []),
    "bp_net_tile_width": (_c_i32, []),
    "bp_net_run": (_c_i32, [_c_ptr, _c_i32, _c_i32, _c_i32, _c_i32, _c_f32, _c_ptr]),
    "bp_net_grid_tile": (_c_i32, [_c_i64]),
    "bp_net_grid_workspace_size": (_c_size, [_c_i64, _c_i32]),
    "bp_net_run_grid": (_c_i32, [_c_ptr, _c_i32, _c_i32, _c_f32, _c_ptr, _c_size, _c_ptr]),
    "bp_net_grid_error": (_c_i32, [_c_ptr, _c_ptr, _c_ptr]),
    "bp_net_grid_cooperative": (_c_i32, []),
    "bp_net_grid_jit_workspace_size": (_c_size, [_c_i64]),
    "bp_net_run_grid_jit": (_c_i32, [_c_ptr, _c_ptr, _c_i32, _c_i32, _c_i32, _c_f32, _c_ptr, _c_size, _c_ptr]),
    "bp_event_csrmv_noalloc_max_rows": (_c_i64, []),
    "bp_event_csrmv_noalloc": (_c_i32, [_c_ptr, _c_i64, _c_ptr, _c_ptr, _c_i32, _c_i64, _c_ptr, _c_i32, _c_i64,
                                        _c_i64, _c_i32, _c_ptr, _c_ptr]),
    "bp_timer_enable": (None, [_c_i32]),
    "bp_timer_collect": (_c_i32, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_c_i64)]),
}


class CsrPlan(ctypes.Structure):
  """Mirror of bp_csr_plan (include/bpgpu.h)."""
  _fields_ = [("m", _c_i64), ("n", _c_i64), ("nnz", _c_i64), ("tile_w", _c_i32), ("n_tiles", _c_i32),
              ("heter", _c_i32), ("variant", _c_i32), ("entries", ctypes.c_uint64), ("mem", _c_ptr),
              ("bytes", _c_size), ("kind", _c_i32)]


class LifParams(ctypes.Structure):
  """Mirror of bp_lif_params (include/bpgpu.h)."""
  _fields_ = [("V_rest", _c_f32), ("V_th", _c_f32), ("V_reset", _c_f32), ("tau", _c_f32), ("tau_ref", _c_f32),
              ("R", _c_f32), ("tau_e", _c_f32), ("tau_i", _c_f32), ("E_e", _c_f32), ("E_i", _c_f32),
              ("input", _c_f32), ("ltc", _c_i32)]


class NetDesc(ctypes.Structure):
  """Mirror of bp_net_desc (include/bpgpu.h)."""
  _fields_ = [("n", _c_i32), ("n_exc", _c_i32), ("tile_w", _c_i32), ("n_tiles", _c_i32),
              ("seg_off", _c_ptr), ("idx", _c_ptr), ("we", _c_f32), ("wi", _c_f32),
              ("p", LifParams), ("V", _c_ptr), ("ge", _c_ptr), ("gi", _c_ptr), ("t_last", _c_ptr),
              ("spike", _c_ptr), ("spike_counts", _c_ptr), ("raster", _c_ptr), ("v_trace", _c_ptr),
              ("trace_steps", _c_i32), ("step_limit", _c_i32), ("step0", _c_i32), ("delay_e", _c_i32),
              ("delay_i", _c_i32), ("ring_len", _c_i32), ("ring", _c_ptr)]


class BPError(RuntimeError):
  pass


def lib():
  """Loads libbpgpu.so (raises if it has not been built)."""
  global _LIB
  if _LIB is None:
    path = _build.LIB
    if not os.path.exists(path):
      raise ImportError(f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()' "
                        "or python -m brainpy_gb300._build); brainpy_gb300 has no fallback compute path")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
      fn = getattr(L, name)
      fn.restype = res
      fn.argtypes = args
    _LIB = L
  return _LIB


def check(status, what):
  if status == BP_OK:
    return
  msg = lib().bp_last_error().decode(errors="replace")
  full = f"{what}: {lib().bp_status_string(status).decode()}: {msg}"
  if status in (BP_ESHAPE, BP_EINVAL):
    raise ValueError(full)
  if status == BP_EDTYPE:
    raise TypeError(full)
  raise BPError(full)


_RAW_STREAM = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def raw_stream(device=None):
  """cudaStream_t (as an int) of the current stream on `device`."""
  if _RAW_STREAM is not None:
    if device is None:
      idx = torch.cuda.current_device()
    elif isinstance(device, torch.device):
      idx = device.index if device.index is not None else torch.cuda.current_device()
    else:
      idx = int(device)
    return _RAW_STREAM(idx)
  return torch.cuda.current_stream(device).cuda_stream


def stream_handle(device=None):
  return ctypes.c_void_p(raw_stream(device))


def ptr(t):
  return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else ctypes.c_void_p(0)


def workspace(nbytes, device):
  return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)
