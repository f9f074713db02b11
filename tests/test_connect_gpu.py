"""FixedProb built on the GPU (bp_fixed_prob_row_lengths / bp_fixed_prob_fill): every row
equal to the oracle's serial restatement of the same generator (bit-exact), for distinct and
multi connections, include_self=False and pre_ratio; at 20,000 x 1e6 with K = 1000, every row
distinct and the columns uniform."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,prob,multi,self_", [(300, 1000, 0.1, False, True), (64, 64, 1.0, False, True),
                                                   (200, 200, 0.3, False, False), (150, 150, 0.2, True, False),
                                                   (100, 5000, 0.02, True, True), (7, 100000, 0.16384, False, True)])
def test_rows_match_oracle(bplib, orc, m, n, prob, multi, self_):
  from brainpy_gb300.connect import FixedProb
  conn = FixedProb(prob, include_self=self_, allow_multi_conn=multi, seed=11)(m, n)
  ind, ptr = conn.require("csr")
  assert ind.dtype == torch.int32 and ptr.dtype == torch.int32 and ptr.numel() == m + 1
  ind, ptr = ind.cpu().numpy(), ptr.cpu().numpy()
  K = int(n * prob)
  rows = orc.fixed_prob_rows(11, range(m), n, K, multi=multi, drop_self=not self_)
  for r in range(m):
    np.testing.assert_array_equal(ind[ptr[r]:ptr[r + 1]], rows[r])


def test_pre_ratio_and_coo(bplib, orc):
  from brainpy_gb300.connect import FixedProb
  m, n = 1000, 300
  conn = FixedProb(0.1, pre_ratio=0.25, seed=4)(m, n)
  ind, ptr = (t.cpu().numpy() for t in conn.require("csr"))
  lens = np.diff(ptr)
  assert (lens > 0).sum() == 250 and set(np.unique(lens)) <= {0, 30}
  sel = np.nonzero(lens)[0]
  rows = orc.fixed_prob_rows(4, sel, n, 30)
  for r, want in zip(sel, rows):
    np.testing.assert_array_equal(ind[ptr[r]:ptr[r + 1]], want)
  pre, post = (t.cpu().numpy() for t in conn.require("coo"))
  np.testing.assert_array_equal(post, ind)
  np.testing.assert_array_equal(pre, np.repeat(np.arange(m), lens))


def test_errors(bplib):
  from brainpy_gb300.connect import FixedProb
  with pytest.raises(ValueError):
    FixedProb(0.1, include_self=False)(10, 20).require("csr")
  with pytest.raises(ValueError):
    FixedProb(1.5)
  from brainpy_gb300 import _lib
  with pytest.raises(_lib.BPError):
    FixedProb(0.5, seed=1)(4, 40000).require("csr")  # 20000 distinct per row > 16384


def test_large_distinct_and_uniform(bplib):
  from brainpy_gb300.connect import FixedProb
  m, n, K = 20000, 1_000_000, 1000
  ind, ptr = FixedProb(K / n, seed=0)(m, n).require("csr")
  assert ind.numel() == m * K
  rows = ind.view(m, K).to(torch.int64)
  s = torch.sort(rows, dim=1).values
  assert bool((s[:, 1:] != s[:, :-1]).all()) and int(s.min()) >= 0 and int(s.max()) < n
  # 2e7 columns over 1e6 bins: chi-square within 6 sigma of its mean
  counts = torch.bincount(rows.reshape(-1), minlength=n).to(torch.float64)
  e = m * K / n
  stat = float(((counts - e) ** 2 / e).sum())
  assert abs(stat - (n - 1)) < 6 * np.sqrt(2 * (n - 1)), stat
  # segment lengths per 27,840-column tile follow the multinomial law (mean 27.84, var ~27.1)
  seg = torch.bincount((rows // 27840 + torch.arange(m, device=rows.device)[:, None] * 36).reshape(-1),
                       minlength=m * 36).view(m, 36)[:, :35].to(torch.float64)
  assert abs(float(seg.mean()) - 27.84) < 0.05 and 24.0 < float(seg.var()) < 30.0


def test_host_device_arrays(bplib):
  """Arrays wanted on the host are built on the GPU and copied; the C entry points refuse
  host output pointers (checked before any launch)."""
  import ctypes
  from brainpy_gb300 import _lib
  from brainpy_gb300.connect import fixed_prob_csr
  ind_c, ptr_c = fixed_prob_csr(300, 500, 20, seed=3, device="cpu")
  ind_g, ptr_g = fixed_prob_csr(300, 500, 20, seed=3)
  assert ind_c.device.type == "cpu" and torch.equal(ind_c, ind_g.cpu()) and torch.equal(ptr_c, ptr_g.cpu())
  host_ind = torch.empty(300 * 20, dtype=torch.int32)
  host_ptr = torch.arange(301, dtype=torch.int64) * 20
  st = _lib.lib().bp_fixed_prob_fill(300, 500, 20, 3, 0, 1, None, ctypes.c_void_p(host_ptr.data_ptr()),
                                     ctypes.c_void_p(host_ind.data_ptr()), None)
  assert st == _lib.BP_EINVAL
