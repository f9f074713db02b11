"""Batched products: a (B, len) batch of vectors through one matrix in one launch pair
(bp_event_csrmv_planned_batch / bp_csrmv_planned_batch), against the oracle row by row.

Bars as for single vectors: homogeneous event counts bit-exact; float sums within 1e-5 of
FP64 scaled by the sum of |terms|."""
import numpy as np
import pytest
import torch

from golden_util import scaled_err

pytestmark = pytest.mark.gpu
TOL = 1e-5
DEV = torch.device("cuda")


def _t(x):
  return torch.as_tensor(x, device=DEV)


def _csr(rng, m, n, kmax, long_row=None):
  lens = rng.integers(0, kmax, m)
  lens[::7] = 0
  if long_row is not None:
    lens[3] = long_row
  ind = np.concatenate([rng.choice(n, l, replace=False) for l in lens]).astype(np.int32)
  ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
  return ind, ptr


@pytest.mark.parametrize("tile_w,cluster", [(512, 1), (512, 4), (None, 4), (None, 2)])
@pytest.mark.parametrize("batch", [1, 3])
def test_plan_batch_against_oracle(bplib, orc, tile_w, cluster, batch):
  from brainpy_gb300.math import event
  rng = np.random.default_rng(31 + batch)
  m, n = 3000, 50001  # n % 4 != 0: output rows after the first are not 16-byte aligned
  ind, ptr = _csr(rng, m, n, 80, long_row=30000)
  heter = rng.normal(size=ind.size).astype(np.float32)
  rates = [0.0, 0.05, 1.0][:batch] if batch > 1 else [0.05]
  ev = np.stack([rng.random(m) < r for r in rates])
  x = (rng.normal(size=(batch, m)) * (rng.random((batch, m)) < 0.5)).astype(np.float32)
  ph = event.prepare(_t(ind), _t(ptr), shape=(m, n), tile_w=tile_w, cluster=cluster)
  pw = event.prepare(_t(ind), _t(ptr), shape=(m, n), data=_t(heter), tile_w=tile_w, cluster=cluster)
  w = _t(np.array([0.75], np.float32))
  yh = ph.csrmv_batch(_t(ev), w).cpu().numpy()
  yw = pw.csrmv_batch(_t(ev)).cpu().numpy()
  sh = ph.sparse_t_batch(_t(x), w).cpu().numpy()
  sw = pw.sparse_t_batch(_t(x)).cpu().numpy()
  assert yh.shape == (batch, n)
  for b in range(batch):
    r = orc.event_csrmv(np.float32(0.75), ind, ptr, ev[b], (m, n), True)
    np.testing.assert_array_equal(yh[b], r["count32"])
    r = orc.event_csrmv(heter, ind, ptr, ev[b], (m, n), True)
    assert scaled_err(yw[b], r["out64"], r["abs64"]) < TOL
    r = orc.csrmv(np.float32(0.75), ind, ptr, x[b], (m, n), True)
    assert scaled_err(sh[b], r["out64"], r["abs64"]) < TOL
    r = orc.csrmv(heter, ind, ptr, x[b], (m, n), True)
    assert scaled_err(sw[b], r["out64"], r["abs64"]) < TOL
    # the batch row equals the single-vector call
    np.testing.assert_array_equal(yh[b], ph.csrmv(_t(ev[b]), w).cpu().numpy())


@pytest.mark.parametrize("transpose", [True, False])
def test_public_batch_functions(bplib, orc, transpose):
  """event.csrmv_batch / sparse.csrmv_batch through the automatic plan (transpose, large
  matrix) and the row-by-row path (transpose=False)."""
  from brainpy_gb300.connect import fixed_prob_csr
  from brainpy_gb300.math import event, sparse
  n, k, batch = 40000, 40, 4
  ind, ptr = fixed_prob_csr(n, n, k, seed=3)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  rng = np.random.default_rng(8)
  ev = rng.random((batch, n)) < 0.03
  x = (rng.normal(size=(batch, n)) * (rng.random((batch, n)) < 0.1)).astype(np.float32)
  y = event.csrmv_batch(0.5, ind, ptr, _t(ev), shape=(n, n), transpose=transpose).cpu().numpy()
  s = sparse.csrmv_batch(-2.0, ind, ptr, _t(x), shape=(n, n), transpose=transpose).cpu().numpy()
  for b in range(batch):
    r = orc.event_csrmv(np.float32(0.5), ind_h, ptr_h, ev[b], (n, n), transpose)
    np.testing.assert_array_equal(y[b], r["count32"])
    r = orc.csrmv(np.float32(-2.0), ind_h, ptr_h, x[b], (n, n), transpose)
    assert scaled_err(s[b], r["out64"], r["abs64"]) < TOL


def test_batch_edge_cases(bplib):
  from brainpy_gb300.math import event
  rng = np.random.default_rng(2)
  m, n = 500, 70000
  ind, ptr = _csr(rng, m, n, 30)
  ph = event.prepare(_t(ind), _t(ptr), shape=(m, n), cluster=4)
  w = _t(np.array([1.0], np.float32))
  y = ph.csrmv_batch(torch.zeros((0, m), dtype=torch.bool, device=DEV), w)
  assert tuple(y.shape) == (0, n)
  with pytest.raises(ValueError):
    ph.csrmv_batch(torch.zeros((2, m + 1), dtype=torch.bool, device=DEV), w)


def test_dnn_layer_batch_matches_rows(bplib):
  from brainpy_gb300 import dnn
  from brainpy_gb300.connect import fixed_prob_csr
  n = 40000
  ind, ptr = fixed_prob_csr(n, n, 30, seed=5)
  layer = dnn.EventCSRLinear((ind, ptr), 0.25, shape=(n, n))
  rng = np.random.default_rng(1)
  x = _t(rng.random((2, 3, n)) < 0.05)
  y = layer(x)
  assert tuple(y.shape) == (2, 3, n)
  for i in range(2):
    for j in range(3):
      assert torch.equal(y[i, j], layer(x[i, j]))
