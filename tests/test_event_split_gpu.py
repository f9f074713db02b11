"""event.csrmv (transpose) on counting plans against the oracle.

A counting plan cuts the columns into tiles of up to 65,472 (16 at N = 1e6), R CTAs per tile
each count a share of the active rows with 16-bit counters, and a second kernel adds the R
partial counts of every column.  Homogeneous weights: bit-exact against the oracle's count form
((float)count * w), including the 32-bit mode a CTA takes when a row holds a column twice or
when its share of active rows exceeds 65,535."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ev(bplib):
  from brainpy_gb300.math import event
  return event


def _events(n, rate, kind, seed):
  rng = np.random.default_rng(seed)
  on = rng.random(n) < rate
  if kind == "bool":
    return on
  vals = rng.normal(0.0, 1.0, n).astype(np.float32)
  vals[~on] = 0.0
  return vals  # float events: > 0 (csrmv) or != 0 (csrmv_taichi) count


def _want(orc, w, ind, ptr, events, shape, rule):
  r = orc.event_csrmv(np.float32(w), ind.cpu().numpy(), ptr.cpu().numpy(), events, shape, True, ev_rule=rule)
  return r["count32"]


def test_count_plan_layout(ev):
  from brainpy_gb300 import _lib
  from brainpy_gb300.connect import fixed_prob_csr
  L = _lib.lib()
  assert L.bp_csr_plan_count_tile(1 << 18) == 0
  tw = L.bp_csr_plan_count_tile(10 ** 6)
  # up to 65,472 columns (16 tiles at N = 1e6): more than twice the general plan's tile
  assert tw % 64 == 0 and tw <= 65_472 and -(-10 ** 6 // tw) == 16
  assert tw > 2 * L.bp_csr_plan_default_tile(10 ** 6, 4)
  ind, ptr = fixed_prob_csr(2000, 600_000, 50, seed=1)
  plan = ev.CSRPlan(ind, ptr, (2000, 600_000), kind="count")
  assert plan.kind == "count" and plan.tile_w == L.bp_csr_plan_count_tile(600_000)
  # weights need the general plan
  w = torch.rand(ind.numel(), device="cuda")
  assert ev.CSRPlan(ind, ptr, (2000, 600_000), data=w, kind="count").kind == "general"


@pytest.mark.parametrize("rate", [0.0, 0.02, 0.5, 1.0])
@pytest.mark.parametrize("kind", ["bool", "float"])
def test_count_plan_matches_oracle(ev, orc, rate, kind):
  from brainpy_gb300.connect import fixed_prob_csr
  m, n, k = 20_000, 600_000, 400
  ind, ptr = fixed_prob_csr(m, n, k, seed=3)
  events = _events(m, rate, kind, seed=4)
  e = torch.as_tensor(events, device="cuda")
  for fn, rule in ((ev.csrmv, orc.EV_F32_POS), (ev.csrmv_taichi, orc.EV_F32_NZ)):
    y = fn(0.75, ind, ptr, e, shape=(m, n), transpose=True).cpu().numpy()
    np.testing.assert_array_equal(y, _want(orc, 0.75, ind, ptr, events, (m, n), rule))
  plan = ev.CSRPlan(ind, ptr, (m, n), kind="count")
  e32 = torch.tensor([0.75], device="cuda")
  np.testing.assert_array_equal(plan.csrmv(e, e32).cpu().numpy(), _want(orc, 0.75, ind, ptr, events, (m, n), orc.EV_F32_POS))
  np.testing.assert_array_equal(plan.csrmv(e, e32, float_rule=2).cpu().numpy(),
                                _want(orc, 0.75, ind, ptr, events, (m, n), orc.EV_F32_NZ))


def test_count_plan_unaligned_output_and_int64(ev, orc):
  from brainpy_gb300.connect import fixed_prob_csr
  m, n, k = 5000, 700_001, 300  # n not a multiple of the tile: the last tile is partial
  ind, ptr = fixed_prob_csr(m, n, k, seed=5, index_dtype=torch.int64)
  events = _events(m, 0.1, "bool", seed=6)
  plan = ev.CSRPlan(ind, ptr, (m, n), kind="count")
  assert plan.kind == "count"
  out = torch.full((n + 1,), -7.0, device="cuda")[1:]  # output 4 bytes past a 16-byte boundary
  y = plan.csrmv(torch.as_tensor(events, device="cuda"), torch.tensor([1.5], device="cuda"), out=out)
  np.testing.assert_array_equal(y.cpu().numpy(), _want(orc, 1.5, ind, ptr, events, (m, n), orc.EV_F32_POS))


def test_count_plan_repeated_columns(ev, orc):
  """Rows that hold a column more than once: the plan records it and every CTA counts in 32
  bits, two passes over its rows (one for each half of the tile)."""
  m, n, k = 3000, 600_000, 300
  g = torch.Generator(device="cpu").manual_seed(7)
  ind = torch.randint(0, n, (m * k,), generator=g, dtype=torch.int32)
  ind.view(m, k)[:, 1] = ind.view(m, k)[:, 0]           # every row repeats a column
  ind.view(m, k)[::7, 2:40] = ind.view(m, k)[::7, :1]   # some rows hold one column 40 times
  ptr = torch.arange(0, m * k + 1, k, dtype=torch.int32)
  ind, ptr = ind.cuda(), ptr.cuda()
  plan = ev.CSRPlan(ind, ptr, (m, n), kind="count")
  assert plan.kind == "count"
  for rate in (0.3, 1.0):
    events = _events(m, rate, "bool", seed=8)
    y = plan.csrmv(torch.as_tensor(events, device="cuda"), torch.tensor([2.0], device="cuda"))
    np.testing.assert_array_equal(y.cpu().numpy(), _want(orc, 2.0, ind, ptr, events, (m, n), orc.EV_F32_POS))


def test_count_plan_many_active_rows(ev, orc):
  """More than 65,535 active rows for one CTA: 32-bit counting, exact."""
  from brainpy_gb300.connect import fixed_prob_csr
  m, n, k = 2_000_000, 600_000, 2
  ind, ptr = fixed_prob_csr(m, n, k, seed=9)
  events = np.ones(m, dtype=bool)
  plan = ev.CSRPlan(ind, ptr, (m, n), kind="count")
  y = plan.csrmv(torch.as_tensor(events, device="cuda"), torch.tensor([1.0], device="cuda"))
  want = _want(orc, 1.0, ind, ptr, events, (m, n), orc.EV_F32_POS)
  np.testing.assert_array_equal(y.cpu().numpy(), want)
  assert float(want.sum()) == m * k


def test_count_plan_rejects_batches_and_vectors(ev):
  from brainpy_gb300 import _lib
  from brainpy_gb300.connect import fixed_prob_csr
  m, n = 1000, 600_000
  ind, ptr = fixed_prob_csr(m, n, 20, seed=10)
  plan = ev.CSRPlan(ind, ptr, (m, n), kind="count")
  e = torch.ones((2, m), dtype=torch.bool, device="cuda")
  with pytest.raises(_lib.BPError, match="one event vector"):
    plan.csrmv_batch(e)
  with pytest.raises(_lib.BPError, match="one event vector"):
    plan.sparse_t(torch.ones(m, device="cuda"))
  # the public batch and dense paths use the general plan of the same matrix
  y = ev.csrmv_batch(1.0, ind, ptr, e, shape=(m, n), transpose=True)
  assert torch.equal(y[0], ev.csrmv(1.0, ind, ptr, e[0], shape=(m, n), transpose=True))
