"""Host-side argument checks of the stored-connectivity and fixed-weight entry points, raised
before any device work (CPU tensors, no GPU)."""
import pytest
import torch


def _cpu_net(**jit):
  from brainpy_gb300 import dyn
  return dyn.EINetwork(100, 80, jitconn=dict(prob=0.1, seeds=(1, 2, 3, 4), **jit), device=torch.device("cpu"))


def test_materialize_takes_the_pull_form_only():
  with pytest.raises(ValueError, match="pull form"):
    _cpu_net(outdim_parallel=False).materialize()


def test_materialize_refuses_stored_connectivity():
  from brainpy_gb300 import dyn
  ind = torch.zeros(0, dtype=torch.int32)
  ptr = torch.zeros(101, dtype=torch.int32)
  net = dyn.EINetwork(100, 80, indices=ind, indptr=ptr, device=torch.device("cpu"))
  with pytest.raises(ValueError, match="already stored"):
    net.materialize()


def test_tune_ops_needs_stored_connectivity():
  with pytest.raises(ValueError, match="stored connectivity"):
    _cpu_net().tune_ops()


@pytest.mark.parametrize("record", [0, 24, 32, 41, 64])
def test_fixed_plan_record_sizes(bplib, record):
  from brainpy_gb300.math import event
  ind = torch.zeros(4, dtype=torch.int32)
  ptr = torch.tensor([0, 2, 4], dtype=torch.int32)
  w = torch.ones(4)
  with pytest.raises(ValueError, match="fix_record"):
    event.CSRPlan(ind, ptr, (2, 3), data=w, kind="fixed", fix_record=record)


def test_fixed_plan_needs_weights(bplib):
  from brainpy_gb300.math import event
  ind = torch.zeros(4, dtype=torch.int32)
  ptr = torch.tensor([0, 2, 4], dtype=torch.int32)
  with pytest.raises(ValueError, match="per-synapse weights"):
    event.CSRPlan(ind, ptr, (2, 3), kind="fixed")
