"""Fixed-weight plans (CSRPlan(kind="fixed"), bp_event_csrmv_planned_fixed): event.csrmv
transpose with per-synapse weights held as int32 fixed point (exact integer shared-memory adds,
out = sum * 2^-k), the weights too small for the fixed point added in float from a side list.
Against the oracle within the 1e-5 bar scaled by the sum of the terms' magnitudes, for weight
laws with and without side entries, both event types and rules, both index types, and at the
benchmarked size."""
import numpy as np
import pytest
import torch

from golden_util import scaled_err

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def ev(bplib):
  from brainpy_gb300.math import event
  return event


def _cmp(ev, orc, plan, w_h, ind_h, ptr_h, events, shape, taichi=False):
  rule = 2 if taichi else 1
  e = torch.as_tensor(events, device="cuda")
  y = plan.csrmv(e, float_rule=rule).cpu().numpy()
  r = orc.event_csrmv(w_h, ind_h, ptr_h, events, shape, True, ev_rule=orc.EV_F32_NZ if taichi else orc.EV_F32_POS)
  assert scaled_err(y, r["out64"], r["abs64"]) < TOL


@pytest.mark.parametrize("law", ["normal_0.5_0.1", "normal_0_1", "wide", "positive"])
def test_fixed_plan_against_oracle(ev, orc, law):
  from brainpy_gb300.connect import fixed_prob_csr
  m, n, k = 60000, 70000, 300
  ind, ptr = fixed_prob_csr(m, n, k, seed=3)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  rng = np.random.default_rng(4)
  nnz = ind_h.size
  if law == "normal_0.5_0.1":
    w = rng.normal(0.5, 0.1, nnz)
  elif law == "normal_0_1":
    w = rng.normal(0.0, 1.0, nnz)           # many weights near zero: a long side list
  elif law == "wide":
    w = rng.choice([-1.0, 1.0], nnz) * 10.0 ** rng.uniform(-9, 3, nnz)  # twelve decades
    w[::97] = 0.0
  else:
    w = rng.uniform(0.5, 1.0, nnz)          # no side entry at all
  w_h = w.astype(np.float32)
  plan = ev.CSRPlan(ind, ptr, (m, n), data=torch.as_tensor(w_h, device="cuda"), kind="fixed")
  assert plan.kind == "fixed" and plan.c.kind == 2
  side = plan.side_entries
  if law == "positive":
    assert side == 0
  if law in ("normal_0_1", "wide"):
    assert side > 0
  for rate in (0.0, 0.02, 1.0):
    _cmp(ev, orc, plan, w_h, ind_h, ptr_h, rng.random(m) < rate, (m, n))
  evf = rng.choice(np.array([0.0, 1.0, -1.0, 0.25], np.float32), m)
  _cmp(ev, orc, plan, w_h, ind_h, ptr_h, evf, (m, n))
  _cmp(ev, orc, plan, w_h, ind_h, ptr_h, evf, (m, n), taichi=True)
  # int64 indices build the same plan
  plan64 = ev.CSRPlan(ind.to(torch.int64), ptr.to(torch.int64), (m, n), data=torch.as_tensor(w_h, device="cuda"),
                      kind="fixed")
  _cmp(ev, orc, plan64, w_h, ind_h, ptr_h, rng.random(m) < 0.1, (m, n))


def test_fixed_plan_full_size(ev, orc):
  """N = 1e6, fan-out 1000, N(0.5, 0.1) weights, 2 % events: the benchmarked heterogeneous
  call on the fixed-weight plan, element-wise against the oracle."""
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr, normal_weights
  n, k = 1_000_000, 1000
  ind, ptr = fixed_prob_csr(n, n, k, seed=0)
  w = normal_weights(ind.numel(), 0.5, 0.1, seed=1)
  plan = ev.CSRPlan(ind, ptr, (n, n), data=w, kind="fixed")
  events = bernoulli_events(n, 0.02, seed=2)
  y = plan.csrmv(events).cpu().numpy()
  r = orc.event_csrmv(w.cpu().numpy(), ind.cpu().numpy(), ptr.cpu().numpy(), events.cpu().numpy(), (n, n), True)
  assert scaled_err(y, r["out64"], r["abs64"]) < TOL
  del plan


def test_fixed_plan_refuses_other_products(ev):
  from brainpy_gb300.connect import fixed_prob_csr
  ind, ptr = fixed_prob_csr(5000, 6000, 50, seed=5)
  w = torch.rand(ind.numel(), device="cuda")
  plan = ev.CSRPlan(ind, ptr, (5000, 6000), data=w, kind="fixed")
  with pytest.raises(Exception):
    plan.csrmv_batch(torch.ones((2, 5000), dtype=torch.bool, device="cuda"))
  with pytest.raises(Exception):
    plan.sparse_n(torch.ones(6000, device="cuda"))
  with pytest.raises(ValueError):
    ev.CSRPlan(ind, ptr, (5000, 6000), kind="fixed")  # needs per-synapse weights


def test_fixed_route_through_public_call(ev, orc, monkeypatch):
  """The "fixed" route (as the autotuner sets it) sends event.csrmv with weights through the
  fixed-weight plan."""
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr
  n, k = 40000, 200
  ind, ptr = fixed_prob_csr(n, n, k, seed=8)
  w = torch.randn(ind.numel(), device="cuda")
  ev.release_plans()
  key = ev._set_route(w, ind, ptr, (n, n), "fixed")
  try:
    events = bernoulli_events(n, 0.05, seed=9)
    y = ev.csrmv(w, ind, ptr, events, shape=(n, n), transpose=True).cpu().numpy()
    assert (ev._matrix_key(w, ind, ptr, n, n), "fixed") in ev._PLANS
    r = orc.event_csrmv(w.cpu().numpy(), ind.cpu().numpy(), ptr.cpu().numpy(), events.cpu().numpy(), (n, n), True)
    assert scaled_err(y, r["out64"], r["abs64"]) < TOL
  finally:
    ev._ROUTES.pop(key, None)
    ev.release_plans()
