"""sparse.csrmv and the CSR utilities on the GPU against the oracle, the golden vectors
(the reference's own Numba kernels) and cuSPARSE (torch's CSR SpMV) as a cross-check."""
import numpy as np
import pytest
import torch

from golden_util import csr_keys, load, scaled_err

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def sp(bplib):
  from brainpy_gb300.math import sparse
  return sparse


def _check(sp, orc, data, ind, ptr, vec, shape, transpose):
  d = torch.as_tensor(np.atleast_1d(data).astype(np.float32), device="cuda")
  y = sp.csrmv(d, torch.as_tensor(ind, device="cuda"), torch.as_tensor(ptr, device="cuda"),
               torch.as_tensor(vec, device="cuda"), shape=shape, transpose=transpose).cpu().numpy()
  r = orc.csrmv(data, ind, ptr, vec, shape, transpose)
  assert scaled_err(y, r["out64"], r["abs64"]) < TOL
  return y


def test_golden_shapes(sp, orc):
  cs = load("csr")
  for key in csr_keys(cs):
    shp, t = key.split("|")
    m, n = (int(x) for x in shp.split("x"))
    transpose = t == "T1"
    ind, ptr = cs[key + "|indices"], cs[key + "|indptr"]
    for wname in ("homo", "heter"):
      if key + f"|sparse_{wname}" not in cs.files:
        continue
      data = np.array([-0.7], np.float32) if wname == "homo" else cs[key + "|heter"]
      y = _check(sp, orc, data, ind, ptr, cs[key + "|vector"], (m, n), transpose)
      r = orc.csrmv(data, ind, ptr, cs[key + "|vector"], (m, n), transpose)
      assert scaled_err(y, cs[key + f"|sparse_{wname}"].astype(np.float64), r["abs64"]) < TOL


@pytest.mark.parametrize("n,k", [(10000, 100), (100000, 300)])
def test_sizes_and_plan(sp, orc, n, k):
  from brainpy_gb300.connect import fixed_prob_csr, normal_weights
  ind, ptr = fixed_prob_csr(n, n, k, seed=3)
  heter = normal_weights(ind.numel(), 0.5, 0.1, seed=4)
  rng = np.random.default_rng(0)
  vec = rng.normal(size=n).astype(np.float32)
  vec[rng.random(n) < 0.5] = 0.0  # zeros are skipped by the transposed kernels
  ih, ph, hh = ind.cpu().numpy(), ptr.cpu().numpy(), heter.cpu().numpy()
  for transpose in (True, False):
    _check(sp, orc, np.float32(0.3), ih, ph, vec, (n, n), transpose)
    _check(sp, orc, hh, ih, ph, vec, (n, n), transpose)


def test_against_cusparse(sp):
  from brainpy_gb300.connect import fixed_prob_csr, normal_weights
  n, k = 50000, 200
  ind, ptr = fixed_prob_csr(n, n, k, seed=5)
  w = normal_weights(ind.numel(), 0.0, 1.0, seed=6)
  x = torch.randn(n, device="cuda")
  A = torch.sparse_csr_tensor(ptr.to(torch.int64), ind.to(torch.int64), w, size=(n, n))
  y_ref = (A @ x.unsqueeze(1)).squeeze(1)
  y = sp.csrmv(w, ind, ptr, x, shape=(n, n), transpose=False)
  scale = (torch.sparse_csr_tensor(ptr.to(torch.int64), ind.to(torch.int64), w.abs(), size=(n, n))
           @ x.abs().unsqueeze(1)).squeeze(1)
  assert float(((y - y_ref).abs() / scale.clamp_min(1e-30)).max()) < 1e-5


def test_utils(sp):
  rng = np.random.default_rng(2)
  m, n = 50, 70
  lens = rng.integers(0, 9, m)
  ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
  ind = np.concatenate([rng.choice(n, l, replace=False) for l in lens]).astype(np.int32)
  data = rng.normal(size=ind.size).astype(np.float32)
  rows, cols = sp.csr_to_coo(torch.as_tensor(ind, device="cuda"), torch.as_tensor(ptr, device="cuda"))
  np.testing.assert_array_equal(rows.cpu().numpy(), np.repeat(np.arange(m), lens))
  dense = sp.csr_to_dense(torch.as_tensor(data, device="cuda"), torch.as_tensor(ind, device="cuda"),
                          torch.as_tensor(ptr, device="cuda"), shape=(m, n)).cpu().numpy()
  expect = np.zeros((m, n), np.float32)
  np.add.at(expect, (np.repeat(np.arange(m), lens), ind), data)
  np.testing.assert_array_equal(dense, expect)
  i2, p2 = sp.coo_to_csr(torch.as_tensor(np.repeat(np.arange(m), lens)[::-1].copy(), device="cuda"),
                         torch.as_tensor(ind[::-1].copy(), device="cuda"), num_row=m)
  np.testing.assert_array_equal(p2.cpu().numpy(), ptr)
  with pytest.raises(ValueError, match="Only support methods"):
    sp.csrmv(1.0, torch.as_tensor(ind, device="cuda"), torch.as_tensor(ptr, device="cuda"),
             torch.ones(n, device="cuda"), shape=(m, n), method="magic")


@pytest.mark.parametrize("tile_w", [512, None])
def test_planned_non_transpose_against_oracle(bplib, orc, tile_w):
  """sparse.csrmv transpose=0 on a plan (column tiles of the vector in shared memory, per-tile
  partial sums added in tile order), homogeneous and heterogeneous, against the FP64 oracle;
  the public call takes the same path through the plan cache."""
  from brainpy_gb300.connect import fixed_prob_csr
  from brainpy_gb300.math import event, sparse
  m, n, k = 3000, 50001, 400
  ind, ptr = fixed_prob_csr(m, n, k, seed=9)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  rng = np.random.default_rng(10)
  x = (rng.normal(size=n) * (rng.random(n) < 0.7)).astype(np.float32)
  heter = rng.normal(size=ind_h.size).astype(np.float32)
  xd = torch.as_tensor(x, device="cuda")
  ph = event.prepare(ind, ptr, shape=(m, n), tile_w=tile_w)
  pw = event.prepare(ind, ptr, shape=(m, n), data=torch.as_tensor(heter, device="cuda"), tile_w=tile_w)
  y = ph.sparse_n(xd, torch.tensor([-1.5], device="cuda")).cpu().numpy()
  r = orc.csrmv(np.float32(-1.5), ind_h, ptr_h, x, (m, n), False)
  assert scaled_err(y, r["out64"], r["abs64"]) < TOL
  y = pw.sparse_n(xd).cpu().numpy()
  r = orc.csrmv(heter, ind_h, ptr_h, x, (m, n), False)
  assert scaled_err(y, r["out64"], r["abs64"]) < TOL
  # the public call: rows of >= 256 entries on average go through the plan cache, shorter
  # rows through the plain row kernel
  m2, n2 = 40000, 40000
  x2 = torch.randn(n2, device="cuda")
  for k2, planned in ((300, True), (60, False)):
    ind2, ptr2 = fixed_prob_csr(m2, n2, k2, seed=2)
    event.release_plans()
    y2 = sparse.csrmv(0.5, ind2, ptr2, x2, shape=(m2, n2), transpose=False).cpu().numpy()
    assert len(event._PLANS) == int(planned)
    r = orc.csrmv(np.float32(0.5), ind2.cpu().numpy(), ptr2.cpu().numpy(), x2.cpu().numpy(), (m2, n2), False)
    assert scaled_err(y2, r["out64"], r["abs64"]) < TOL
  event.release_plans()
