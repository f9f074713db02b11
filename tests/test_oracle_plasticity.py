"""The oracle's STDP weight updates and CSR -> CSC conversion against the golden fixtures
generated from the reference's own source (brainpy/_src/dnn/linear.py:650-698,
brainpy/_src/connect/base.py:645-726): bit-exact."""
import numpy as np

from golden_util import load

BOUNDS = [(-np.inf, np.inf), (-0.1, 0.6), (0.0, 0.3)]


def _cases(g):
  return sorted({k.split("|")[0] for k in g.files})


def test_plasticity_oracle_matches_golden(orc):
  g = load("plasticity")
  for key in _cases(g):
    m, n = (int(x) for x in key.split("x"))
    ind, ptr, w = g[key + "|indices"], g[key + "|indptr"], g[key + "|w"]
    pre, cptr, wid = orc.csr2csc(ind, ptr, n)
    np.testing.assert_array_equal(pre, g[key + "|csc_pre_ids"])
    np.testing.assert_array_equal(cptr, g[key + "|csc_indptr"])
    np.testing.assert_array_equal(wid, g[key + "|csc_w_ids"])
    for bi, (lo, hi) in enumerate(BOUNDS):
      r = orc.csr_on_pre_update(w, ind, ptr, g[key + "|pre_spike"], g[key + "|post_trace"], lo, hi)
      np.testing.assert_array_equal(r.view(np.uint32), g[key + f"|on_pre|{bi}"].view(np.uint32))
      r = orc.csc_on_post_update(w, g[key + "|csc_pre_ids"], g[key + "|csc_indptr"], g[key + "|csc_w_ids"],
                                 g[key + "|post_spike"], g[key + "|pre_trace"], lo, hi)
      np.testing.assert_array_equal(r.view(np.uint32), g[key + f"|on_post|{bi}"].view(np.uint32))


def test_plasticity_oracle_nan_and_float_spikes(orc):
  """numpy's minimum/maximum keep NaN; a float spike counts when nonzero (Python truth)."""
  ind = np.array([0, 1, 2, 0], np.int32)
  ptr = np.array([0, 3, 4], np.int32)
  w = np.array([0.1, 0.2, 0.3, 0.4], np.float32)
  trace = np.array([np.nan, 1.0, -5.0], np.float32)
  r = orc.csr_on_pre_update(w, ind, ptr, np.array([-0.5, 0.0], np.float32), trace, -1.0, 1.0)
  assert np.isnan(r[0]) and r[1] == 1.0 and r[2] == -1.0 and r[3] == np.float32(0.4)
