"""Autotuning support: timing candidates, firing-rate buckets, and a persistent choice cache.

The event-driven transpose product has two kernel families for one matrix: the row-parallel
kernel (one warp per active row, global atomics; no setup) and the column-tiled plan (one
cluster per column tile, shared-memory accumulation; a one-time plan build), the latter in
several variants (lanes per segment, chunk rounds, extra-chunk prefetch).  Which is fastest
depends on the matrix (rows, columns, fan-out, weights) and on the firing rate.
``brainpy_gb300.math.event.autotune`` times them on a representative spike vector and keeps
the winner per matrix; this module holds the parts that do not touch the GPU:

* ``rate_bucket``: firing rates grouped in half-octaves, so that a choice made at 2 % serves
  every rate in [1.86 %, 2.63 %);
* ``make_key``: the cache key (device name, operator, sizes, weight kind, event type, bucket);
* ``TuneCache``: choices kept in memory and, when a path is given (argument or the
  ``BPGPU_TUNE_CACHE`` environment variable), in a JSON file, so a later process reuses them
  without timing again;
* ``pick``: times every candidate with a supplied timer and returns the fastest.
"""
import json
import math
import os
import tempfile
from typing import Callable, Dict, Optional, Tuple

CACHE_VERSION = 1


def rate_bucket(rate: float) -> float:
  """Half-octave bucket of a firing rate in (0, 1]: round(2 log2 rate) / 2.  Zero and
  negative rates share the bucket -inf (reported as the string "none" in keys)."""
  if not rate > 0.0:
    return float("-inf")
  return round(2.0 * math.log2(min(rate, 1.0))) / 2.0


def make_key(op: str, device: str, m: int, n: int, nnz: int, heter: bool, etype: int, bucket: float) -> str:
  b = "none" if bucket == float("-inf") else f"{bucket:+.1f}"
  return f"{op}|{device}|m={int(m)}|n={int(n)}|nnz={int(nnz)}|{'heter' if heter else 'homo'}|e={int(etype)}|r={b}"


class TuneCache:
  """Tuning records by key; persisted as JSON when a path is set.  A file written by another
  cache version, or one that does not parse, is ignored (and replaced on the next save)."""

  def __init__(self, path: Optional[str] = None):
    self.path = path
    self.entries: Dict[str, dict] = {}
    if path:
      self.load()

  def load(self):
    try:
      with open(self.path) as f:
        blob = json.load(f)
    except (OSError, ValueError):
      return
    if isinstance(blob, dict) and blob.get("version") == CACHE_VERSION and isinstance(blob.get("entries"), dict):
      self.entries.update(blob["entries"])

  def lookup(self, key: str) -> Optional[dict]:
    return self.entries.get(key)

  def store(self, key: str, record: dict):
    self.entries[key] = dict(record)

  def save(self):
    """Writes the file atomically (a temporary file in the same folder, then a rename)."""
    if not self.path:
      return
    folder = os.path.dirname(os.path.abspath(self.path))
    os.makedirs(folder, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=".tune-", suffix=".json", dir=folder)
    try:
      with os.fdopen(fd, "w") as f:
        json.dump({"version": CACHE_VERSION, "entries": self.entries}, f, indent=1, sort_keys=True)
      os.replace(tmp, self.path)
    except BaseException:
      if os.path.exists(tmp):
        os.unlink(tmp)
      raise


_DEFAULT: Optional[TuneCache] = None


def default_cache() -> TuneCache:
  """The process-wide cache: memory only, or backed by the file ``$BPGPU_TUNE_CACHE``."""
  global _DEFAULT
  if _DEFAULT is None:
    _DEFAULT = TuneCache(os.environ.get("BPGPU_TUNE_CACHE") or None)
  return _DEFAULT


def pick(candidates: Dict[str, Callable[[], object]], timer: Callable[[Callable[[], object]], float]
         ) -> Tuple[str, Dict[str, float]]:
  """Times every candidate (``timer(fn)`` returns microseconds per call) and returns the name
  of the fastest with all the times.  Ties go to the candidate listed first."""
  if not candidates:
    raise ValueError("pick: no candidates")
  times = {name: float(timer(fn)) for name, fn in candidates.items()}
  best = min(times, key=lambda k: (times[k], list(candidates).index(k)))
  return best, times


def cuda_timer(reps: int = 10, warmup: int = 2):
  """A timer for ``pick``: CUDA events around ``reps`` back-to-back calls on the current
  stream, after ``warmup`` untimed calls; microseconds per call."""
  import torch

  def timer(fn):
    for _ in range(warmup):
      fn()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(reps):
      fn()
    t1.record()
    t1.synchronize()
    return t0.elapsed_time(t1) * 1e3 / reps

  return timer
