"""bench.py's host helpers without a GPU: the algorithmic-byte formula of the headline
roofline (spikes, indptr pairs, int32 indices, float32 weights, float32 output) and the
result comparison used by its self-checks."""
import os
import sys

import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_algorithmic_bytes_headline():
  n, k, active = 1_000_000, 1000, 20_000  # N = 1e6, K = 1000, 2 % of rows active
  homo = bench.alg_bytes(n, active, k, False)
  heter = bench.alg_bytes(n, active, k, True)
  assert homo == n + 8 * active + 4 * active * k + 4 * n == 85_160_000
  assert heter - homo == 4 * active * k
  # 60 % of the measured peak at these bytes is the 20.9 us bar
  assert abs(homo / (0.6 * 6803.8e9) * 1e6 - 20.86) < 0.01


def test_same_result_exact_and_tolerant():
  a = torch.tensor([1.0, 2.0, 3.0])
  assert bench.same_result(a, a.clone(), heter=False)
  b = a.clone()
  b[1] = torch.nextafter(b[1], torch.tensor(10.0))
  assert not bench.same_result(a, b, heter=False)  # homogeneous: bit for bit
  assert bench.same_result(a, b, heter=True)  # weighted: within 1e-5 of the largest magnitude
  c = a.clone()
  c[0] += 1e-3
  assert not bench.same_result(a, c, heter=True)
  z = torch.zeros(3)
  assert bench.same_result(z, z.clone(), heter=True)


def test_profile_traffic_read_from_committed_summaries():
  """The `traffic` key of the roofline comes from the committed ncu summaries: the headline
  kernel's 53.0 MB a call and the weighted path's 123.0 MB (40-byte fixed-weight records)."""
  assert bench.profile_traffic("event_csrmv_N1e6_K1000_rate2pct_homo.md") == 53_000_000
  assert bench.profile_traffic("event_csrmv_N1e6_K1000_rate2pct_heter.md") == 123_000_000
  assert bench.profile_traffic("no_such_summary.md") is None
