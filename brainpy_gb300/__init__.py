"""brainpy_gb300 -- GB300-native (sm_103a) event-driven synaptic propagation with
BrainPy's operator interface.

  brainpy_gb300.math.event.csrmv / csrmv_taichi / info
  brainpy_gb300.math.sparse.csrmv / csrmv_taichi / csr_to_dense
  brainpy_gb300.math.jitconn.{event_,}mv_prob_{homo,uniform,normal}[_taichi]
  brainpy_gb300.dyn (LIF/COBA network state update and runners)

All compute runs in libbpgpu.so (hand-written CUDA for sm_103a, C ABI declared in
include/bpgpu.h).  Arrays are torch tensors on a CUDA device.
"""
from . import _build  # noqa: F401

__version__ = "0.1.0"


def build(force=False, verbose=False):
  """Compiles libbpgpu.so in tree (nvcc, sm_103a)."""
  return _build.build_library(force=force, verbose=verbose)
