"""The C ABI library: it loads, exports every symbol include/bpgpu.h declares, and its
host-side validation rejects bad arguments before touching the GPU (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
  names = []
  for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
    if not h.endswith(".h"):
      continue
    src = open(os.path.join(ROOT, "include", h)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names += re.findall(r"^[A-Za-z_][\w \*]*?\b(bp_\w+)\s*\(", src, flags=re.M)
  return sorted(set(names))


def test_header_declares_entry_points():
  names = header_functions()
  assert "bp_event_csrmv" in names and "bp_event_info" in names
  assert len(names) >= 8


def test_library_exports_every_declared_symbol(bplib):
  missing = [n for n in header_functions() if not hasattr(bplib, n)]
  assert not missing, missing


def test_python_binding_covers_header(bplib):
  from brainpy_gb300 import _lib
  missing = [n for n in header_functions() if n not in _lib.SIGNATURES]
  assert not missing, missing


def test_status_strings(bplib):
  from brainpy_gb300 import _lib
  assert bplib.bp_status_string(_lib.BP_OK) == b"BP_OK"
  assert b"shape" in bplib.bp_status_string(_lib.BP_ESHAPE)
  assert bplib.bp_version() >= 0x000100


def _call_event_csrmv(L, **kw):
  from brainpy_gb300 import _lib
  a = dict(data=1, ndata=1, indices=1, indptr=1, itype=_lib.BP_I32, nnz=10, events=1, etype=_lib.BP_EV_BOOL,
           m=4, n=5, transpose=1, out=1, ws=1, ws_bytes=1 << 20, stream=None)
  a.update(kw)
  p = lambda v: ctypes.c_void_p(v) if v else ctypes.c_void_p(0)
  return L.bp_event_csrmv(p(a["data"]), a["ndata"], p(a["indices"]), p(a["indptr"]), a["itype"], a["nnz"],
                          p(a["events"]), a["etype"], a["m"], a["n"], a["transpose"], p(a["out"]), p(a["ws"]),
                          a["ws_bytes"], p(a["stream"]))


def test_host_validation_without_gpu(bplib):
  from brainpy_gb300 import _lib
  assert _call_event_csrmv(bplib, m=-1) == _lib.BP_EINVAL
  assert _call_event_csrmv(bplib, ndata=3) == _lib.BP_ESHAPE
  assert b"consistent with indices" in bplib.bp_last_error()
  assert _call_event_csrmv(bplib, itype=7) == _lib.BP_EDTYPE
  assert _call_event_csrmv(bplib, etype=9) == _lib.BP_EDTYPE
  assert _call_event_csrmv(bplib, out=0) == _lib.BP_EINVAL
  assert _call_event_csrmv(bplib, ws_bytes=8) == _lib.BP_ENOMEM
  assert bplib.bp_event_info(None, 0, -3, None, ctypes.c_void_p(1), None, 0, None) == _lib.BP_EINVAL


def test_workspace_sizes(bplib):
  assert bplib.bp_event_csrmv_workspace_size(1000, 10, 0) == 0
  assert bplib.bp_event_csrmv_workspace_size(1000, 10, 1) >= 4 * 1000
  assert bplib.bp_event_info_workspace_size(10 ** 6) >= 4 * (10 ** 6 // 4096)


def test_front_end_fails_loudly_without_library(monkeypatch, tmp_path):
  from brainpy_gb300 import _build, _lib
  monkeypatch.setattr(_build, "LIB", str(tmp_path / "missing.so"))
  monkeypatch.setattr(_lib, "_LIB", None)
  with pytest.raises(ImportError, match="no fallback"):
    _lib.lib()
