import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)


def pytest_configure(config):
  config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_ok():
  try:
    import torch
    return torch.cuda.is_available()
  except Exception:
    return False


def pytest_collection_modifyitems(config, items):
  if _cuda_ok():
    return
  skip = pytest.mark.skip(reason="no CUDA device")
  for it in items:
    if "gpu" in it.keywords:
      it.add_marker(skip)


@pytest.fixture(scope="session")
def orc():
  import oracle
  oracle.build()
  return oracle


@pytest.fixture(scope="session")
def bplib():
  """libbpgpu.so built in tree (nvcc cross-compiles, no GPU needed)."""
  import brainpy_gb300
  brainpy_gb300.build()
  from brainpy_gb300 import _lib
  return _lib.lib()
