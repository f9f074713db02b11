"""Autotuner host logic without a GPU: rate buckets, cache keys, the JSON choice cache
(round trip, foreign versions, corrupt files), candidate picking with a supplied timer, and
the per-matrix routes that make later csrmv calls skip or force the tiled plan."""
import gc
import json

import pytest
import torch

from brainpy_gb300 import tuning


def test_rate_bucket_half_octaves():
  # 2 % shares its bucket with [2^-5.75, 2^-5.25) = [1.86 %, 2.63 %)
  assert tuning.rate_bucket(0.02) == tuning.rate_bucket(0.019) == tuning.rate_bucket(0.026)
  assert tuning.rate_bucket(0.018) != tuning.rate_bucket(0.02) != tuning.rate_bucket(0.027)
  assert tuning.rate_bucket(0.02) != tuning.rate_bucket(0.1)
  assert tuning.rate_bucket(0.005) < tuning.rate_bucket(0.02) < tuning.rate_bucket(0.1) < tuning.rate_bucket(1.0)
  assert tuning.rate_bucket(1.0) == 0.0 and tuning.rate_bucket(2.0) == 0.0
  assert tuning.rate_bucket(0.0) == float("-inf") == tuning.rate_bucket(-1.0)
  assert tuning.rate_bucket(0.5) == -1.0


def test_keys_separate_every_field():
  base = dict(op="event_csrmv_T", device="GB300", m=10, n=20, nnz=30, heter=False, etype=0, bucket=-5.5)
  k0 = tuning.make_key(**base)
  for field, other in (("op", "x"), ("device", "B200"), ("m", 11), ("n", 21), ("nnz", 31), ("heter", True),
                       ("etype", 1), ("bucket", -5.0)):
    assert tuning.make_key(**dict(base, **{field: other})) != k0, field
  assert "r=none" in tuning.make_key(**dict(base, bucket=float("-inf")))


def test_cache_round_trip(tmp_path):
  path = tmp_path / "sub" / "tune.json"
  c = tuning.TuneCache(str(path))
  assert c.lookup("k") is None
  c.store("k", {"choice": "tiled:514", "times_us": {"row": 50.0, "tiled:514": 31.0}, "rate": 0.02})
  c.save()
  blob = json.loads(path.read_text())
  assert blob["version"] == tuning.CACHE_VERSION and "k" in blob["entries"]
  again = tuning.TuneCache(str(path))
  assert again.lookup("k")["choice"] == "tiled:514"
  assert [p.name for p in path.parent.iterdir()] == ["tune.json"]  # no temporary file left


def test_cache_ignores_foreign_or_corrupt_files(tmp_path):
  p = tmp_path / "tune.json"
  p.write_text(json.dumps({"version": tuning.CACHE_VERSION + 1, "entries": {"k": {"choice": "row"}}}))
  assert tuning.TuneCache(str(p)).lookup("k") is None
  p.write_text("{not json")
  c = tuning.TuneCache(str(p))
  assert c.entries == {}
  c.store("k", {"choice": "row"})
  c.save()
  assert tuning.TuneCache(str(p)).lookup("k") == {"choice": "row"}


def test_memory_only_cache_does_not_write(tmp_path, monkeypatch):
  monkeypatch.chdir(tmp_path)
  c = tuning.TuneCache()
  c.store("k", {"choice": "row"})
  c.save()
  assert list(tmp_path.iterdir()) == []


def test_pick_fastest_with_supplied_timer():
  calls = []
  cands = {name: (lambda name=name: calls.append(name)) for name in ("row", "tiled:258", "tiled:260")}
  fake = {"row": 80.0, "tiled:258": 31.0, "tiled:260": 35.0}
  order = iter(["row", "tiled:258", "tiled:260"])

  def timer(fn):
    fn()
    return fake[next(order)]

  best, times = tuning.pick(cands, timer)
  assert best == "tiled:258" and times == fake and calls == ["row", "tiled:258", "tiled:260"]
  # ties go to the candidate listed first
  best, _ = tuning.pick({"a": lambda: None, "b": lambda: None}, lambda fn: 1.0)
  assert best == "a"
  with pytest.raises(ValueError):
    tuning.pick({}, lambda fn: 0.0)


def test_routes_skip_or_force_the_plan(bplib):
  from brainpy_gb300.math import event as ev
  indices = torch.zeros(8, dtype=torch.int32)
  indptr = torch.zeros(5, dtype=torch.int32)
  data = torch.ones(1)
  shape = (4, 1 << 20)
  key = ev._set_route(data, indices, indptr, shape, "row")
  try:
    assert ev._route(data, indices, indptr, shape) == "row"
    # a "row" route returns no plan, whatever the size thresholds say (nothing is built)
    assert ev._cached_plan(data, indices, indptr, shape) is None
    # an in-place change of the indices invalidates the route
    indices.add_(0)
    assert ev._route(data, indices, indptr, shape) is None
  finally:
    ev._ROUTES.pop(key, None)
  # a route whose arrays are gone is dropped on lookup
  idx2 = torch.zeros(8, dtype=torch.int32)
  key2 = ev._set_route(data, idx2, indptr, shape, "tiled")
  del idx2
  gc.collect()
  ent = ev._ROUTES.get(key2)
  assert ent is not None and ent[0][0]() is None
  ev._ROUTES.pop(key2, None)


def test_valid_choices(bplib):
  from brainpy_gb300.math import event as ev
  codes = ev.CSRPlan.variants()
  assert codes and ev._valid_choice("row") and ev._valid_choice("split")
  assert all(ev._valid_choice(f"tiled:{c}") for c in codes)
  for bad in ("tiled:999999", "tiled:x", "columns", None, 3):
    assert not ev._valid_choice(bad)


def test_net_tile_candidates_and_classes(bplib):
  from brainpy_gb300 import dyn
  L = bplib
  tmax, cap = L.bp_net_max_tiles(), L.bp_net_tile_width()
  assert dyn.tile_candidates(1000) == [1024, 2048, 4096]
  # a network may not need more CTAs than a cluster holds
  n_big = tmax * 2048 + 1
  assert dyn.tile_candidates(n_big) == [t for t in (4096,) if t <= cap]
  assert dyn.tile_candidates(1000, (1000, 64, cap + 64)) == [64]
  assert dyn.size_class(4000) == dyn.size_class(4200) != dyn.size_class(6000)
  assert dyn.size_class(1) == 0.0
