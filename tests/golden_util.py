"""Access to the committed golden fixtures (generated by tests/golden/make_golden.py
from the reference's own kernel source)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
  return np.load(os.path.join(GOLDEN, name + ".npz"))


def jitconn_keys(g):
  return sorted({k.rsplit("|", 1)[0] for k in g.files})


def csr_keys(g):
  return sorted({k.rsplit("|", 1)[0] for k in g.files if not k.startswith("info")})


def scaled_err(y, y64, abs64):
  """max |y - y64| / max(|y64|, sum|terms|) -- the FP32-vs-FP64 bar (1e-5)."""
  y = np.asarray(y, np.float64)
  scale = np.maximum(np.abs(y64), abs64)
  err = np.abs(y - y64)
  if err.size == 0:
    return 0.0
  ok = scale > 0
  worst = np.max(err[ok] / scale[ok]) if ok.any() else 0.0
  if (~ok).any():
    worst = max(worst, float(np.max(err[~ok])))
  return float(worst)
