"""event.csrmv / event.info on the GPU against the oracle and the golden vectors.

Bars: homogeneous weights -> bit-exact against the oracle's count form ((float)count*w);
every case -> within 1e-5 of the FP64 sum, scaled by max(|y|, sum|terms|)."""
import numpy as np
import pytest
import torch

from golden_util import csr_keys, load, scaled_err

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def ev(bplib):
  from brainpy_gb300.math import event
  return event


def _check(ev, orc, data, ind, ptr, events, shape, transpose, taichi=False):
  dev = torch.device("cuda")
  fn = ev.csrmv_taichi if taichi else ev.csrmv
  d = torch.as_tensor(np.atleast_1d(data).astype(np.float32), device=dev)
  y = fn(d, torch.as_tensor(ind, device=dev), torch.as_tensor(ptr, device=dev), torch.as_tensor(events, device=dev),
         shape=shape, transpose=transpose).cpu().numpy()
  r = orc.event_csrmv(data, ind, ptr, events, shape, transpose, ev_rule=orc.EV_F32_NZ if taichi else orc.EV_F32_POS)
  assert y.dtype == np.float32 and y.shape == r["out64"].shape
  assert scaled_err(y, r["out64"], r["abs64"]) < TOL
  if r["count32"] is not None:
    np.testing.assert_array_equal(y, r["count32"])
  return y


def test_golden_shapes(ev, orc):
  cs = load("csr")
  for key in csr_keys(cs):
    shp, t = key.split("|")
    m, n = (int(x) for x in shp.split("x"))
    transpose = t == "T1"
    ind, ptr = cs[key + "|indices"], cs[key + "|indptr"]
    for wname in ("homo", "heter"):
      if key + f"|event_bool_{wname}" not in cs.files:
        continue
      data = np.array([-0.7], np.float32) if wname == "homo" else cs[key + "|heter"]
      for kind, events in (("event_bool", cs[key + "|events"]), ("event_float", cs[key + "|events_f"])):
        y = _check(ev, orc, data, ind, ptr, events, (m, n), transpose)
        # and against the reference's own outputs (golden), FP32 within tolerance
        ref = cs[key + f"|{kind}_{wname}"]
        r = orc.event_csrmv(data, ind, ptr, events, (m, n), transpose)
        assert scaled_err(y, ref.astype(np.float64), r["abs64"]) < TOL


@pytest.mark.parametrize("n,k", [(10000, 100), (10000, 1000), (100000, 100), (100000, 1000)])
@pytest.mark.parametrize("rate", [0.005, 0.02, 0.1])
def test_config_sweep_sizes(ev, orc, n, k, rate):
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr, normal_weights
  ind, ptr = fixed_prob_csr(n, n, k, seed=0)
  events = bernoulli_events(n, rate, seed=2).cpu().numpy()
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  _check(ev, orc, np.float32(1.0), ind_h, ptr_h, events, (n, n), True)
  heter = normal_weights(ind.numel(), 0.5, 0.1, seed=1).cpu().numpy()
  _check(ev, orc, heter, ind_h, ptr_h, events, (n, n), True)
  if n <= 10000:
    _check(ev, orc, np.float32(0.6), ind_h, ptr_h, events, (n, n), False)
    _check(ev, orc, heter, ind_h, ptr_h, events, (n, n), False)


def test_edge_cases(ev, orc):
  rng = np.random.default_rng(5)
  m, n = 300, 200
  lens = rng.integers(0, 40, m)
  lens[::7] = 0  # empty rows
  ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
  ind = np.concatenate([rng.permutation(n)[:l] for l in lens]).astype(np.int32)
  heter = rng.normal(size=ind.size).astype(np.float32)
  for events in (np.zeros(m, bool), np.ones(m, bool), rng.random(m) < 0.5):
    for data in (np.float32(2.5), heter):
      _check(ev, orc, data, ind, ptr, events, (m, n), True)
  # int64 indices
  _check(ev, orc, heter, ind.astype(np.int64), ptr.astype(np.int64), rng.random(m) < 0.3, (m, n), True)
  # float events: negatives and zeros are not events under the `> 0` rule, are under `!= 0`
  evf = rng.choice(np.array([0.0, 1.0, -1.0, 0.25], np.float32), m)
  _check(ev, orc, heter, ind, ptr, evf, (m, n), True)
  _check(ev, orc, heter, ind, ptr, evf, (m, n), True, taichi=True)
  # unaligned event vector (a slice starting at an odd byte)
  big = torch.as_tensor(rng.random(m + 1) < 0.4, device="cuda")
  sl = big[1:]
  y = ev.csrmv(1.0, torch.as_tensor(ind, device="cuda"), torch.as_tensor(ptr, device="cuda"), sl,
               shape=(m, n), transpose=True).cpu().numpy()
  r = orc.event_csrmv(np.float32(1.0), ind, ptr, sl.cpu().numpy(), (m, n), True)
  np.testing.assert_array_equal(y, r["count32"])
  # empty matrix
  y = ev.csrmv(1.0, torch.zeros(0, dtype=torch.int32, device="cuda"), torch.zeros(5, dtype=torch.int32, device="cuda"),
               torch.ones(4, dtype=torch.bool, device="cuda"), shape=(4, 9), transpose=True)
  assert y.shape == (9,) and float(y.abs().sum()) == 0.0


@pytest.mark.parametrize("m,n,k", [
    (3200, 4000, 80),     # the COBA example's excitatory rows: one round of the single-CTA kernel
    (20000, 3000, 20),    # several rounds of event scanning (4096 events a round)
    (5000, 49152, 100),   # the largest output held in shared memory
    (5000, 49153, 100),   # one column more: the general path
    (600, 4000, 900),     # 540K entries: the one-cluster kernel
    (20000, 30000, 200),  # 4M entries, 20K rows: the one-cluster kernel
    (270000, 2000, 4),    # more rows than the cluster scans: the general path
])
def test_small_single_launch_path(ev, orc, m, n, k):
  """The single-launch kernels of transposed products with a small output (all columns in
  shared memory: one CTA, or one cluster whose CTAs split the rows and sum through
  distributed shared memory) and the general path on either side of their limits agree with
  the oracle: bit-exact counts for a homogeneous weight, the FP64 bar for heterogeneous
  weights, every event rule and both index types."""
  from brainpy_gb300.connect import fixed_prob_csr, normal_weights
  ind, ptr = fixed_prob_csr(m, n, k, seed=4)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  heter = normal_weights(ind.numel(), 0.5, 0.1, seed=5).cpu().numpy()
  rng = np.random.default_rng(6)
  for rate in (0.0, 0.02, 1.0):
    events = rng.random(m) < rate
    _check(ev, orc, np.float32(0.6), ind_h, ptr_h, events, (m, n), True)
    _check(ev, orc, heter, ind_h, ptr_h, events, (m, n), True)
  evf = rng.choice(np.array([0.0, 1.0, -1.0, 0.25], np.float32), m)
  _check(ev, orc, np.float32(-1.5), ind_h, ptr_h, evf, (m, n), True)
  _check(ev, orc, heter, ind_h, ptr_h, evf, (m, n), True, taichi=True)
  _check(ev, orc, heter, ind_h.astype(np.int64), ptr_h.astype(np.int64), rng.random(m) < 0.1, (m, n), True)


def test_shape_errors(ev):
  ind = torch.zeros(4, dtype=torch.int32, device="cuda")
  ptr = torch.tensor([0, 2, 4], dtype=torch.int32, device="cuda")
  with pytest.raises(ValueError, match="Shape mismatch"):
    ev.csrmv(1.0, ind, ptr, torch.ones(3, dtype=torch.bool, device="cuda"), shape=(2, 5), transpose=True)
  with pytest.raises(ValueError, match="consistent with indices"):
    ev.csrmv(torch.ones(3, device="cuda"), ind, ptr, torch.ones(2, dtype=torch.bool, device="cuda"), shape=(2, 5),
             transpose=True)
  with pytest.raises(ValueError, match="int32 or int64"):
    ev.csrmv(1.0, ind.to(torch.int16), ptr, torch.ones(2, dtype=torch.bool, device="cuda"), shape=(2, 5),
             transpose=True)


def test_info(ev, orc):
  cs = load("csr")
  for n in (1, 5, 100, 1000, 4097):
    e = cs[f"info|{n}|events"]
    ids, num = ev.info(torch.as_tensor(e, device="cuda"))
    np.testing.assert_array_equal(ids.cpu().numpy(), cs[f"info|{n}|ids"])
    assert int(num.cpu()[0]) == int(cs[f"info|{n}|num"][0])
  rng = np.random.default_rng(1)
  for n in (4096 * 37 + 5, 10 ** 6):
    e = rng.random(n) < 0.02
    ids, num = ev.info(torch.as_tensor(e, device="cuda"))
    rid, rnum = orc.event_info(e)
    np.testing.assert_array_equal(ids.cpu().numpy(), rid)
    assert int(num.cpu()[0]) == rnum


def test_full_size_properties(ev):
  """N = 1e6, fan-out 1000, 2 % events: size-independent identities.
  (a) homo output / w is the exact integer count, summing to the number of events;
  (b) linearity in the event set: disjoint halves add up exactly (integer counts)."""
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr
  n, k = 10 ** 6, 1000
  ind, ptr = fixed_prob_csr(n, n, k, seed=0)
  events = bernoulli_events(n, 0.02, seed=2)
  y = ev.csrmv(1.0, ind, ptr, events, shape=(n, n), transpose=True)
  n_events = int(events.sum()) * k
  assert float(y.double().sum()) == n_events
  assert torch.equal(y, torch.round(y))
  half = torch.zeros_like(events)
  half[: n // 2] = events[: n // 2]
  y1 = ev.csrmv(1.0, ind, ptr, half, shape=(n, n), transpose=True)
  y2 = ev.csrmv(1.0, ind, ptr, events & ~half, shape=(n, n), transpose=True)
  assert torch.equal(y1 + y2, y)
  y3 = ev.csrmv(0.37, ind, ptr, events, shape=(n, n), transpose=True)
  assert torch.equal(y3, y * np.float32(0.37))


def test_full_size_against_oracle(ev, orc):
  """The benchmark configuration (N = 1e6, fan-out 1000, 2 % events) element by element
  against the oracle: a homogeneous weight bit-exact (the counting plan, 16-bit counters),
  per-synapse weights within the 1e-5 bar (the general plan)."""
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr, normal_weights
  n, k = 10 ** 6, 1000
  ind, ptr = fixed_prob_csr(n, n, k, seed=0)
  events = bernoulli_events(n, 0.02, seed=2)
  ind_h, ptr_h, ev_h = ind.cpu().numpy(), ptr.cpu().numpy(), events.cpu().numpy()
  y = ev.csrmv(0.6, ind, ptr, events, shape=(n, n), transpose=True)
  r = orc.event_csrmv(np.float32(0.6), ind_h, ptr_h, ev_h, (n, n), True)
  np.testing.assert_array_equal(y.cpu().numpy(), r["count32"])
  heter = normal_weights(ind.numel(), 0.5, 0.1, seed=1)
  y = ev.csrmv(heter, ind, ptr, events, shape=(n, n), transpose=True).cpu().numpy()
  r = orc.event_csrmv(heter.cpu().numpy(), ind_h, ptr_h, ev_h, (n, n), True)
  assert scaled_err(y, r["out64"], r["abs64"]) < TOL
  del heter
  ev.release_plans()


@pytest.mark.parametrize("cluster", [1, 2, 4, 8])
def test_tiled_plan_clusters(ev, orc, cluster):
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr, normal_weights
  n, k = 100000, 300
  ind, ptr = fixed_prob_csr(n, n, k, seed=4)
  heter = normal_weights(ind.numel(), 0.5, 0.1, seed=5)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  for tile_w in (None, 1024, 4000):
    plan_h = ev.prepare(ind, ptr, shape=(n, n), tile_w=tile_w, cluster=cluster)
    plan_w = ev.prepare(ind, ptr, shape=(n, n), data=heter, tile_w=tile_w, cluster=cluster)
    for rate in (0.005, 0.1, 1.0):
      events = bernoulli_events(n, rate, seed=6)
      ev_h = events.cpu().numpy()
      y = plan_h.csrmv(events, torch.tensor([0.25], device="cuda")).cpu().numpy()
      r = orc.event_csrmv(np.float32(0.25), ind_h, ptr_h, ev_h, (n, n), True)
      np.testing.assert_array_equal(y, r["count32"])
      y = plan_w.csrmv(events).cpu().numpy()
      r = orc.event_csrmv(heter.cpu().numpy(), ind_h, ptr_h, ev_h, (n, n), True)
      assert scaled_err(y, r["out64"], r["abs64"]) < TOL


def test_tiled_plan_irregular_rows(ev, orc):
  """Rows of uneven length (incl. empty and very long), int64 indices, n not a multiple
  of the tile, unaligned output."""
  rng = np.random.default_rng(9)
  m, n = 5000, 70001
  lens = rng.integers(0, 60, m)
  lens[::11] = 0
  lens[5] = 20000
  ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
  ind = np.concatenate([rng.choice(n, l, replace=False) for l in lens]).astype(np.int64)
  heter = rng.normal(size=ind.size).astype(np.float32)
  ind_d, ptr_d = torch.as_tensor(ind, device="cuda"), torch.as_tensor(ptr, device="cuda")
  for tile_w in (64, 3000, None):
    plan = ev.prepare(ind_d, ptr_d, shape=(m, n), tile_w=tile_w, cluster=2)
    planw = ev.prepare(ind_d, ptr_d, shape=(m, n), data=torch.as_tensor(heter, device="cuda"), tile_w=tile_w,
                       cluster=4)
    for events in (np.ones(m, bool), rng.random(m) < 0.3, np.zeros(m, bool)):
      e = torch.as_tensor(events, device="cuda")
      big = torch.zeros(n + 1, device="cuda")
      out = big[1:]  # 4-byte aligned but not 16-byte aligned
      plan.csrmv(e, torch.tensor([1.5], device="cuda"), out=out)
      r = orc.event_csrmv(np.float32(1.5), ind, ptr, events, (m, n), True)
      np.testing.assert_array_equal(out.cpu().numpy(), r["count32"])
      y = planw.csrmv(e).cpu().numpy()
      r = orc.event_csrmv(heter, ind, ptr, events, (m, n), True)
      assert scaled_err(y, r["out64"], r["abs64"]) < TOL


def test_plan_cache_and_rowpar_agree(ev, orc, monkeypatch):
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr
  n, k = 100000, 200
  ind, ptr = fixed_prob_csr(n, n, k, seed=7)
  events = bernoulli_events(n, 0.02, seed=8)
  y_plan = ev.csrmv(0.5, ind, ptr, events, shape=(n, n), transpose=True)
  assert len(ev._PLANS) >= 1
  monkeypatch.setattr(ev, "_PLAN_DISABLE", True)
  y_row = ev.csrmv(0.5, ind, ptr, events, shape=(n, n), transpose=True)
  assert torch.equal(y_plan, y_row)
  monkeypatch.setattr(ev, "_PLAN_DISABLE", False)
  n_before = len(ev._PLANS)
  ind.add_(0)  # in-place write bumps the version counter -> the plan is rebuilt in place
  y2 = ev.csrmv(0.5, ind, ptr, events, shape=(n, n), transpose=True)
  assert len(ev._PLANS) == n_before and torch.equal(y2, y_plan)


@pytest.mark.parametrize("variant", ["1,1,0", "2,1,1", "4,1,0", "2,2,1", "8,1,1", "8,2,0"])
def test_tiled_kernel_variants(bplib, orc, variant):
  """The planned kernels in every compiled variant (lanes per segment, chunk rounds, L1
  prefetch of a segment's extra chunks), on rows of uneven length including one far longer than a round.  Runs in a
  child process (the variant is read once per process)."""
  import os
  import subprocess
  import sys
  env = dict(os.environ, BPGPU_TILED=variant)
  here = os.path.dirname(os.path.abspath(__file__))
  r = subprocess.run([sys.executable, os.path.join(here, "_tiled_case.py")], env=env, capture_output=True, text=True,
                     timeout=600)
  assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-2000:] + r.stderr[-4000:]


def test_plan_autotune_and_every_variant(ev, orc):
  """The plan's autotuner times every compiled variant and keeps the fastest; every variant
  gives the oracle's exact counts."""
  from brainpy_gb300.connect import fixed_prob_csr
  n, k = 50000, 200
  ind, ptr = fixed_prob_csr(n, n, k, seed=4)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  rng = np.random.default_rng(6)
  events = rng.random(n) < 0.05
  plan = ev.prepare(ind, ptr, shape=(n, n))
  w = torch.tensor([0.5], device="cuda")
  e = torch.as_tensor(events, device="cuda")
  times = plan.autotune(e, w, reps=3)
  assert set(times) == set(plan.variants()) and plan.variant == min(times, key=times.get)
  want = orc.event_csrmv(np.float32(0.5), ind_h, ptr_h, events, (n, n), True)["count32"]
  for code in plan.variants():
    plan.variant = code
    np.testing.assert_array_equal(plan.csrmv(e, w).cpu().numpy(), want)
  plan.variant = 3 | 3 << 8  # not a compiled variant
  from brainpy_gb300 import _lib
  with pytest.raises(_lib.BPError):
    plan.csrmv(e, w)


def test_autotune_routes_row_or_tiled(ev, orc, tmp_path):
  """event.autotune times the row-parallel kernel against every tiled variant, keeps the
  winner for the matrix, and later csrmv calls follow it; a cached record is applied without
  timing (a forced "row" record means no plan is held); results are the oracle's counts."""
  from brainpy_gb300 import tuning
  from brainpy_gb300.connect import fixed_prob_csr
  n, k = 40000, 100  # below the plan size thresholds: untuned calls take the row kernel
  ind, ptr = fixed_prob_csr(n, n, k, seed=9)
  rng = np.random.default_rng(10)
  events = rng.random(n) < 0.02
  e = torch.as_tensor(events, device="cuda")
  w = torch.tensor([0.5], device="cuda")
  want = orc.event_csrmv(np.float32(0.5), ind.cpu().numpy(), ptr.cpu().numpy(), events, (n, n), True)["count32"]
  cache = tuning.TuneCache(str(tmp_path / "tune.json"))
  rec = ev.autotune(w, ind, ptr, e, shape=(n, n), cache=cache, reps=3)
  codes = ev.CSRPlan.variants()
  assert set(rec["times_us"]) == {"row"} | {f"tiled:{c}" for c in codes}
  assert rec["choice"] == min(rec["times_us"], key=rec["times_us"].get)
  assert abs(rec["rate"] - events.mean()) < 1e-12
  key = ev._matrix_key(w, ind, ptr, n, n)
  assert ev._ROUTES[key][2] == rec["choice"].split(":")[0]
  assert ((key, "general") in ev._PLANS) == rec["choice"].startswith("tiled")
  np.testing.assert_array_equal(ev.csrmv(w, ind, ptr, e, shape=(n, n), transpose=True).cpu().numpy(), want)
  # the record was saved; a fresh cache reads it, and a forced record is applied as is
  again = tuning.TuneCache(str(tmp_path / "tune.json"))
  assert len(again.entries) == 1
  (rk, _), = again.entries.items()
  for forced in ["tiled:" + str(codes[0]), "row"]:
    again.store(rk, {"choice": forced, "times_us": {}, "rate": rec["rate"]})
    got = ev.autotune(w, ind, ptr, e, shape=(n, n), cache=again)
    assert got["choice"] == forced and got["times_us"] == {}
    assert ev._ROUTES[key][2] == forced.split(":")[0]
    assert ((key, "general") in ev._PLANS) == (forced != "row")
    if forced != "row":
      assert ev._PLANS[(key, "general")][2].variant == codes[0]
    np.testing.assert_array_equal(ev.csrmv(w, ind, ptr, e, shape=(n, n), transpose=True).cpu().numpy(), want)
    np.testing.assert_array_equal(
        ev.csrmv_batch(w, ind, ptr, e[None], shape=(n, n), transpose=True)[0].cpu().numpy(), want)
  # transpose=False has one family: nothing is timed
  assert ev.autotune(w, ind, ptr, e, shape=(n, n), transpose=False)["choice"] == "row"
  ev._ROUTES.pop(key, None)


@pytest.mark.parametrize("n,evkind", [(200_000, "bool"), (1_000_000, "float"), (2_000_000, "bool")])
def test_non_transpose_bits_path(ev, orc, n, evkind):
  """transpose=0 with the event vector as bits in shared memory (n <= 1.6M), and beyond it
  the per-entry gather kernel: counts bit-exact, weights within the FP32 bar."""
  from brainpy_gb300.connect import fixed_prob_csr
  m, k = 50_000, 300
  ind, ptr = fixed_prob_csr(m, n, k, seed=12)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  rng = np.random.default_rng(13)
  mask = rng.random(n) < 0.05
  events = mask if evkind == "bool" else (rng.normal(size=n) * mask).astype(np.float32)
  e = torch.as_tensor(events, device="cuda")
  y = ev.csrmv(0.25, ind, ptr, e, shape=(m, n), transpose=False).cpu().numpy()
  r = orc.event_csrmv(np.float32(0.25), ind_h, ptr_h, events, (m, n), False)
  np.testing.assert_array_equal(y, r["count32"])
  heter = rng.normal(size=ind_h.size).astype(np.float32)
  y = ev.csrmv(torch.as_tensor(heter, device="cuda"), ind, ptr, e, shape=(m, n), transpose=False).cpu().numpy()
  r = orc.event_csrmv(heter, ind_h, ptr_h, events, (m, n), False)
  assert scaled_err(y, r["out64"], r["abs64"]) < TOL
