"""STDP weight updates of the CSR layers on the GPU (bp_csr_on_pre_update,
bp_csc_on_post_update) and the CSC conversion, against the golden fixtures from the
reference's source and the oracle: bit-exact (one float32 add and a clip per update)."""
import numpy as np
import pytest
import torch

from golden_util import load

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
BOUNDS = [(-np.inf, np.inf), (-0.1, 0.6), (0.0, 0.3)]


def _t(x):
  return torch.as_tensor(x, device=DEV)


def _bits(x):
  return np.asarray(x, np.float32).view(np.uint32)


def test_golden(bplib):
  from brainpy_gb300 import dnn
  from brainpy_gb300.connect import csr2csc
  g = load("plasticity")
  for key in sorted({k.split("|")[0] for k in g.files}):
    m, n = (int(x) for x in key.split("x"))
    ind, ptr, w = g[key + "|indices"], g[key + "|indptr"], g[key + "|w"]
    pre, cptr, wid = csr2csc(_t(ind), _t(ptr), n)
    np.testing.assert_array_equal(pre.cpu().numpy(), g[key + "|csc_pre_ids"])
    np.testing.assert_array_equal(cptr.cpu().numpy(), g[key + "|csc_indptr"])
    np.testing.assert_array_equal(wid.cpu().numpy(), g[key + "|csc_w_ids"])
    for bi, (lo, hi) in enumerate(BOUNDS):
      wt = _t(w)
      r = dnn.csr_on_pre_update(wt, _t(ind), _t(ptr), _t(g[key + "|pre_spike"]), _t(g[key + "|post_trace"]), lo, hi)
      np.testing.assert_array_equal(_bits(r.cpu()), _bits(g[key + f"|on_pre|{bi}"]))
      assert torch.equal(wt, _t(w))  # the functional form leaves its input alone
      r = dnn.csc_on_post_update(wt, pre, cptr, wid, _t(g[key + "|post_spike"]), _t(g[key + "|pre_trace"]), lo, hi)
      np.testing.assert_array_equal(_bits(r.cpu()), _bits(g[key + f"|on_post|{bi}"]))


@pytest.mark.parametrize("itype", [np.int32, np.int64])
@pytest.mark.parametrize("float_spikes", [False, True])
def test_large_against_oracle_and_in_place(bplib, orc, itype, float_spikes):
  from brainpy_gb300 import dnn
  from brainpy_gb300.connect import csr2csc, fixed_prob_csr
  m = n = 20000
  ind, ptr = fixed_prob_csr(m, n, 100, seed=7, index_dtype=torch.int32 if itype == np.int32 else torch.int64)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  rng = np.random.default_rng(3)
  w = rng.normal(0.5, 0.2, ind_h.size).astype(np.float32)
  if float_spikes:
    pre_sp = (rng.normal(size=m) * (rng.random(m) < 0.05)).astype(np.float32)
    post_sp = (rng.normal(size=n) * (rng.random(n) < 0.05)).astype(np.float32)
  else:
    pre_sp, post_sp = rng.random(m) < 0.05, rng.random(n) < 0.05
  post_tr = rng.normal(0, 0.1, n).astype(np.float32)
  pre_tr = rng.normal(0, 0.1, m).astype(np.float32)
  want = orc.csr_on_pre_update(w, ind_h, ptr_h, pre_sp, post_tr, 0.0, 1.0)
  wt = _t(w)
  dnn.csr_on_pre_update(wt, ind, ptr, _t(pre_sp), _t(post_tr), 0.0, 1.0, out=wt)
  np.testing.assert_array_equal(_bits(wt.cpu()), _bits(want))
  cpre, cptr, cwid = orc.csr2csc(ind_h, ptr_h, n)
  pre, c_indptr, wid = csr2csc(ind, ptr, n)
  np.testing.assert_array_equal(pre.cpu().numpy(), cpre)
  np.testing.assert_array_equal(wid.cpu().numpy(), cwid)
  want2 = orc.csc_on_post_update(want, cpre, cptr, cwid, post_sp, pre_tr, 0.0, 1.0)
  dnn.csc_on_post_update(wt, pre, c_indptr, wid, _t(post_sp), _t(pre_tr), 0.0, 1.0, out=wt)
  np.testing.assert_array_equal(_bits(wt.cpu()), _bits(want2))


def test_nan_and_edges(bplib, orc):
  from brainpy_gb300 import dnn
  ind = np.array([0, 1, 2, 0, 9], np.int32)  # 9 >= n: never updated
  ptr = np.array([0, 3, 5], np.int32)
  w = np.array([0.1, 0.2, 0.3, 0.4, 0.5], np.float32)
  trace = np.array([np.nan, 1.0, -5.0], np.float32)
  sp = np.array([-0.5, 2.0], np.float32)
  r = dnn.csr_on_pre_update(_t(w), _t(ind), _t(ptr), _t(sp), _t(trace), -1.0, 1.0).cpu().numpy()
  assert np.isnan(r[0]) and r[1] == 1.0 and r[2] == -1.0 and np.isnan(r[3]) and r[4] == np.float32(0.5)
  empty = dnn.csr_on_pre_update(_t(np.zeros(0, np.float32)), _t(np.zeros(0, np.int32)), _t(np.zeros(3, np.int32)),
                                _t(np.ones(2, bool)), _t(trace))
  assert empty.numel() == 0


def test_layer_stdp_update(bplib, orc):
  from brainpy_gb300 import dnn
  from brainpy_gb300.connect import fixed_prob_csr
  m, n = 3000, 2000
  ind, ptr = fixed_prob_csr(m, n, 50, seed=1)
  rng = np.random.default_rng(9)
  w0 = rng.normal(0.5, 0.1, ind.numel()).astype(np.float32)
  layer = dnn.EventCSRLinear((ind, ptr), _t(w0.copy()), shape=(m, n))
  pre_sp, post_sp = rng.random(m) < 0.1, rng.random(n) < 0.1
  pre_tr, post_tr = rng.normal(0, 0.1, m).astype(np.float32), rng.normal(0, 0.1, n).astype(np.float32)
  layer.stdp_update(on_pre={"spike": _t(pre_sp), "trace": _t(post_tr)},
                    on_post={"spike": _t(post_sp), "trace": _t(pre_tr)}, w_min=0.0, w_max=1.0)
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  want = orc.csr_on_pre_update(w0, ind_h, ptr_h, pre_sp, post_tr, 0.0, 1.0)
  cpre, cptr, cwid = orc.csr2csc(ind_h, ptr_h, n)
  want = orc.csc_on_post_update(want, cpre, cptr, cwid, post_sp, pre_tr, 0.0, 1.0)
  np.testing.assert_array_equal(_bits(layer.weight.cpu()), _bits(want))
  with pytest.raises(ValueError):
    dnn.EventCSRLinear((ind, ptr), 0.5, shape=(m, n)).stdp_update(on_pre={"spike": _t(pre_sp), "trace": _t(post_tr)})


def test_stdp_loop_keeps_one_plan(bplib):
  """In-place STDP updates bump the weights' version counter; the plan cache replaces the
  layer's plan instead of keeping one per version, so device memory stays flat over steps."""
  from brainpy_gb300 import dnn
  from brainpy_gb300.connect import fixed_prob_csr
  from brainpy_gb300.math import event as ev
  n, k = 40_000, 40  # above the plan thresholds (n >= 32768 columns, nnz >= 2^20)
  ind, ptr = fixed_prob_csr(n, n, k, seed=11)
  layer = dnn.EventCSRLinear((ind, ptr), torch.full((ind.numel(),), 0.5, device="cuda"), shape=(n, n))
  ev.release_plans()
  rng = np.random.default_rng(12)
  spikes = _t(rng.random(n) < 0.05)
  trace = _t(rng.normal(0, 0.01, n).astype(np.float32))
  mem = []
  for _ in range(6):
    layer.update(spikes)
    layer.stdp_update(on_pre={"spike": spikes, "trace": trace}, w_min=0.0, w_max=1.0)
    torch.cuda.synchronize()
    mem.append(torch.cuda.memory_allocated())
  assert len(ev._PLANS) == 1
  assert mem[-1] == mem[1], mem
  ev.release_plans()
