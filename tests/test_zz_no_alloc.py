"""bp_event_csrmv_noalloc: event.csrmv for callers that cannot allocate.

A legacy XLA custom-call target (how the reference binds its operators) is handed only its
operand and result buffers, with no scratch allocator, and may not cudaMalloc mid-stream.
This entry point keeps its scratch in a fixed device array inside the library.  Checked
here through the C ABI against bp_event_csrmv (caller-provided workspace): bit-exact for
homogeneous weights, within the 1e-5 scaled FP64 bar for heterogeneous ones, on two calls
in a row with different spike vectors (the shared scratch must not leak between calls).
This file is collected last on purpose; it also runs alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _vp(t):
  return ctypes.c_void_p(t.data_ptr())


@pytest.fixture(scope="module")
def L(bplib):
  return bplib


def _workload(n, k, seed):
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr, normal_weights
  ind, ptr = fixed_prob_csr(n, n, k, seed=seed)
  heter = normal_weights(ind.numel(), 0.5, 0.1, seed=seed + 1)
  return ind, ptr, heter, [bernoulli_events(n, r, seed=seed + 2 + j) for j, r in enumerate((0.02, 0.1))]


def _events(ev, etype):
  """bool events, or float32 events of both signs (the > 0 and != 0 rules then differ)."""
  from brainpy_gb300 import _lib
  if etype == _lib.BP_EV_BOOL:
    return ev.view(torch.uint8)
  sign = torch.where(torch.arange(ev.numel(), device=ev.device) % 3 == 0, -1.0, 1.0)
  return ev.to(torch.float32) * sign


def _with_workspace(L, data, ind, ptr, ev, n, transpose, etype=0, itype=0):
  out = torch.full((n,), float("nan"), device="cuda")
  ws_bytes = L.bp_event_csrmv_workspace_size(n, n, transpose)
  ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device="cuda")
  st = L.bp_event_csrmv(_vp(data), data.numel(), _vp(ind), _vp(ptr), itype, ind.numel(),
                        _vp(ev), etype, n, n, transpose, _vp(out), _vp(ws), ws_bytes,
                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
  assert st == 0, L.bp_last_error()
  return out


def _no_alloc(L, data, ind, ptr, ev, n, transpose, etype=0, itype=0):
  out = torch.full((n,), float("nan"), device="cuda")
  st = L.bp_event_csrmv_noalloc(_vp(data), data.numel(), _vp(ind), _vp(ptr), itype, ind.numel(),
                                _vp(ev), etype, n, n, transpose, _vp(out),
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
  assert st == 0, L.bp_last_error()
  return out


def _scaled_err(y, ref, terms):
  y, ref, terms = (t.double().cpu().numpy() for t in (y, ref, terms))
  scale = np.maximum(np.abs(ref), terms)
  return float(np.max(np.abs(y - ref) / np.maximum(scale, 1e-30)))


@pytest.mark.parametrize("etype", [0, 1, 2])  # BP_EV_BOOL, BP_EV_F32_POS, BP_EV_F32_NZ
@pytest.mark.parametrize("itype", [0, 1])      # BP_I32, BP_I64
def test_matches_workspace_entry_point_twice(L, etype, itype):
  n, k = 20000, 100
  ind, ptr, heter, spikes = _workload(n, k, seed=11)
  if itype == 1:
    ind, ptr = ind.to(torch.int64), ptr.to(torch.int64)
  homo = torch.tensor([0.6], device="cuda")
  for transpose in (1, 0):
    for ev in spikes:  # two calls in a row on different events
      e = _events(ev, etype)
      a = _no_alloc(L, homo, ind, ptr, e, n, transpose, etype, itype)
      b = _with_workspace(L, homo, ind, ptr, e, n, transpose, etype, itype)
      torch.cuda.synchronize()
      assert torch.equal(a, b)
      a = _no_alloc(L, heter, ind, ptr, e, n, transpose, etype, itype)
      b = _with_workspace(L, heter, ind, ptr, e, n, transpose, etype, itype)
      terms = _with_workspace(L, heter.abs(), ind, ptr, e, n, transpose, etype, itype)
      torch.cuda.synchronize()
      assert _scaled_err(a, b, terms) < 1e-5


def test_rejects_rows_beyond_the_limit(L):
  from brainpy_gb300 import _lib
  limit = L.bp_event_csrmv_noalloc_max_rows()
  assert limit >= 1 << 20
  dummy = ctypes.c_void_p(16)
  st = L.bp_event_csrmv_noalloc(dummy, 1, dummy, dummy, _lib.BP_I32, 10, dummy, _lib.BP_EV_BOOL, limit + 1, 5, 1,
                                dummy, None)
  assert st == _lib.BP_ENOMEM
  assert b"scratch limit" in L.bp_last_error()
