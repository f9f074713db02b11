"""Fixed-weight plans (CSRPlan(kind="fixed"), bp_event_csrmv_planned_fixed): event.csrmv
transpose with per-synapse weights held as int32 fixed point (exact integer shared-memory adds,
out = sum * 2^-k), the weights too small for the fixed point added in float from a side list.
Against the oracle within the 1e-5 bar scaled by the sum of the terms' magnitudes, for weight
laws with and without side entries, both event types and rules, both index types, and at the
benchmarked size; the 40-byte chunk records (24-bit weights) against the 48-byte ones (int32)."""
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
  assert plan.fix_record == 40  # N(0.5, 0.1) at fan-in ~1000: the weights fit 24 bits
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


def _plan_chunks(plan):
  """The plan's own chunks: a mask of those that belong to a segment (the plan leaves unused
  gaps between rows; row r's segments are chunks [seg_off[r][0], seg_off[r][T])), and every
  chunk's 8 indices and 8 integer weights (the plan's weight array after the conversion)."""
  import ctypes
  from brainpy_gb300 import _lib
  so_p, idx_p, w_p = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
  _lib.check(_lib.lib().bp_csr_plan_arrays(ctypes.byref(plan.c), ctypes.byref(so_p), ctypes.byref(idx_p),
                                           ctypes.byref(w_p)), "csr_plan_arrays")
  m, t = plan.shape[0], int(plan.c.n_tiles)
  nch = int(plan.c.entries) // 8
  mem = plan.mem.cpu().numpy()
  base = plan.mem.data_ptr()

  def arr(p, nbytes, dtype):
    off = p.value - base
    return mem[off:off + nbytes].view(dtype)

  so = arr(so_p, 4 * m * (t + 1), np.uint32).reshape(m, t + 1).astype(np.int64)
  d = np.zeros(nch + 1, np.int64)
  np.add.at(d, so[:, 0], 1)
  np.add.at(d, so[:, t], -1)
  seg = np.cumsum(d)[:nch] > 0
  return seg, arr(idx_p, 16 * nch, np.uint16).reshape(nch, 8), arr(w_p, 32 * nch, np.int32).reshape(nch, 8)


def _decode48(fx, nchunks):
  """(indices, integer weights) of every chunk from 48-byte records."""
  rec = fx[:48 * nchunks].reshape(nchunks, 48)
  return rec[:, :16].copy().view(np.uint16), rec[:, 16:].copy().view(np.int32)


def _decode40(fx, nchunks):
  """(indices, integer weights) of every chunk from 40-byte records: an even chunk holds its
  indices, the low 16 bits of its weights and their high bytes; an odd one the high bytes first."""
  rec = fx[:40 * nchunks].reshape(nchunks, 40)
  odd = (np.arange(nchunks) & 1).astype(bool)[:, None]
  idx = np.where(odd, rec[:, 8:24], rec[:, 0:16]).copy().view(np.uint16)
  lo = np.where(odd, rec[:, 24:40], rec[:, 16:32]).copy().view(np.uint16).astype(np.int64)
  hi = np.where(odd, rec[:, 0:8], rec[:, 32:40]).copy().view(np.int8).astype(np.int64)
  return idx, (hi * 65536 + lo).astype(np.int32)


@pytest.mark.parametrize("law", ["normal_0.5_0.1", "positive", "normal_0_1"])
def test_fixed_records_40_and_48(ev, orc, law):
  """At fan-in ~1000, N(0.5, 0.1) and U[0.5, 1] weights fit 24 bits and take 40-byte records by
  default; each plan's records (40 or 48 bytes) hold that plan's indices and integer weights, and
  the two forms give the same results (bit for bit without side entries).  N(0, 1) weights reach more than
  256 times a column's mean: 48-byte records, and 40 is refused."""
  from brainpy_gb300.connect import fixed_prob_csr
  m = n = 20000
  ind, ptr = fixed_prob_csr(m, n, 1000, seed=11)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  rng = np.random.default_rng(12)
  nnz = ind_h.size
  if law == "normal_0.5_0.1":
    w_h = rng.normal(0.5, 0.1, nnz).astype(np.float32)
  elif law == "positive":
    w_h = rng.uniform(0.5, 1.0, nnz).astype(np.float32)
  else:
    w_h = rng.normal(0.0, 1.0, nnz).astype(np.float32)
  w = torch.as_tensor(w_h, device="cuda")
  plan = ev.CSRPlan(ind, ptr, (m, n), data=w, kind="fixed")
  plan48 = ev.CSRPlan(ind, ptr, (m, n), data=w, kind="fixed", fix_record=48)
  assert plan48.fix_record == 48
  if law == "normal_0_1":
    assert plan.fix_record == 48
    with pytest.raises(ValueError):
      ev.CSRPlan(ind, ptr, (m, n), data=w, kind="fixed", fix_record=40)
    return
  assert plan.fix_record == 40
  # each plan's records hold its own chunks (two builds may order a segment's entries apart)
  for p, decode in ((plan, _decode40), (plan48, _decode48)):
    seg, idx, q = _plan_chunks(p)
    assert seg.sum() * 8 >= nnz
    ridx, rq = decode(p.fx.cpu().numpy(), idx.shape[0])
    assert np.array_equal(ridx[seg], idx[seg]) and np.array_equal(rq[seg], q[seg])
  if law == "positive":
    assert plan.side_entries == 0
  for rate in (0.0, 0.02, 0.3, 1.0):
    e = torch.as_tensor(rng.random(m) < rate, device="cuda")
    y40, y48 = plan.csrmv(e), plan48.csrmv(e)
    if law == "positive":
      assert torch.equal(y40, y48)
    r = orc.event_csrmv(w_h, ind_h, ptr_h, e.cpu().numpy(), (m, n), True)
    assert scaled_err(y40.cpu().numpy(), r["out64"], r["abs64"]) < TOL
    assert scaled_err(y48.cpu().numpy(), r["out64"], r["abs64"]) < TOL
