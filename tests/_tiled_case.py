"""Child process of test_tiled_kernel_variants: runs the planned event/sparse kernels in the
variant given in BPGPU_TILED and checks them against the oracle, fixed-weight plans with both
chunk record sizes included.  Prints OK."""
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from golden_util import scaled_err  # noqa: E402

from brainpy_gb300.math import event  # noqa: E402
import oracle  # noqa: E402


def main():
  oracle.build()
  orc = oracle
  rng = np.random.default_rng(21)
  m, n = 3000, 50001
  lens = rng.integers(0, 80, m)
  lens[::7] = 0
  lens[3] = 30000  # one row far longer than one round of chunks
  ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
  ind = np.concatenate([rng.choice(n, l, replace=False) for l in lens]).astype(np.int32)
  heter = rng.normal(size=ind.size).astype(np.float32)
  dev = torch.device("cuda")
  ind_d, ptr_d = torch.as_tensor(ind, device=dev), torch.as_tensor(ptr, device=dev)
  # fixed-weight plans: a hub column (column 0 first in every nonempty row, a duplicate where the
  # row also drew it) makes the largest column sum of |w| ~2000, so that N(0, 1) weights fit 24
  # bits; ~8 % of them fall below tau and go to the side list
  ind_f = ind.copy()
  ind_f[ptr[:-1][lens > 0]] = 0
  ind_fd = torch.as_tensor(ind_f, device=dev)
  heter_d = torch.as_tensor(heter, device=dev)
  for tile_w in (512, None):
    for cluster in (1, 4):
      ph = event.prepare(ind_d, ptr_d, shape=(m, n), tile_w=tile_w, cluster=cluster)
      pw = event.prepare(ind_d, ptr_d, shape=(m, n), data=torch.as_tensor(heter, device=dev), tile_w=tile_w,
                         cluster=cluster)
      for rate in (0.0, 0.05, 1.0):
        ev = rng.random(m) < rate
        e = torch.as_tensor(ev, device=dev)
        y = ph.csrmv(e, torch.tensor([0.75], device=dev)).cpu().numpy()
        r = orc.event_csrmv(np.float32(0.75), ind, ptr, ev, (m, n), True)
        np.testing.assert_array_equal(y, r["count32"])
        y = pw.csrmv(e).cpu().numpy()
        r = orc.event_csrmv(heter, ind, ptr, ev, (m, n), True)
        assert scaled_err(y, r["out64"], r["abs64"]) < 1e-5
        x = (rng.normal(size=m) * (rng.random(m) < max(rate, 0.5))).astype(np.float32)
        xd = torch.as_tensor(x, device=dev)
        y = ph.sparse_t(xd, torch.tensor([0.75], device=dev)).cpu().numpy()
        r = orc.csrmv(np.float32(0.75), ind, ptr, x, (m, n), True)
        assert scaled_err(y, r["out64"], r["abs64"]) < 1e-5
        y = pw.sparse_t(xd, None).cpu().numpy()
        r = orc.csrmv(heter, ind, ptr, x, (m, n), True)
        assert scaled_err(y, r["out64"], r["abs64"]) < 1e-5
      for rec in (40, 48):
        pf = event.CSRPlan(ind_fd, ptr_d, (m, n), data=heter_d, tile_w=tile_w, cluster=cluster, kind="fixed",
                           fix_record=rec)
        assert pf.fix_record == rec and pf.side_entries > 0
        for rate in (0.0, 0.05, 1.0):
          ev = rng.random(m) < rate
          y = pf.csrmv(torch.as_tensor(ev, device=dev)).cpu().numpy()
          r = orc.event_csrmv(heter, ind_f, ptr, ev, (m, n), True)
          assert scaled_err(y, r["out64"], r["abs64"]) < 1e-5
  print("OK")


if __name__ == "__main__":
  main()
