"""The FixedProb generator's algorithm on the oracle (no GPU): the law of the reference's
rng.choice(post_num, K, replace=False) per row (brainpy/_src/connect/random_conn.py:73-128).
Rows are the first K distinct values of a counter-based i.i.d. uniform sequence: checked
here for exact size, distinctness, range, uniform marginals and uniform first position."""
import numpy as np


def _chi2_ok(counts, expected, dof):
  """Chi-square statistic within 6 standard deviations of its mean (dof)."""
  stat = float(np.sum((counts - expected) ** 2 / expected))
  return abs(stat - dof) < 6.0 * np.sqrt(2.0 * dof), stat


def test_rows_distinct_exact_in_range(orc):
  for n, K in [(1000, 100), (64, 64), (5, 1), (100000, 1000)]:
    rows = orc.fixed_prob_rows(7, range(50), n, K)
    for r in rows:
      assert r.size == K and np.unique(r).size == K and r.min() >= 0 and r.max() < n


def test_marginals_and_order_uniform(orc):
  n, K, m = 50, 10, 4000
  rows = np.stack(orc.fixed_prob_rows(3, range(m), n, K))
  ok, stat = _chi2_ok(np.bincount(rows.ravel(), minlength=n), m * K / n, n - 1)
  assert ok, stat
  ok, stat = _chi2_ok(np.bincount(rows[:, 0], minlength=n), m / n, n - 1)  # the first position too
  assert ok, stat


def test_multi_and_self(orc):
  n, K = 20, 10
  rows = orc.fixed_prob_rows(5, range(2000), n, K, multi=True)
  assert all(r.size == K for r in rows)
  repeats = np.mean([K - np.unique(r).size for r in rows])
  want = K - n * (1 - (1 - 1 / n) ** K)  # expected repeats of K uniform draws out of n
  assert abs(repeats - want) < 0.15
  rows = orc.fixed_prob_rows(5, range(n), n, K, drop_self=True)
  full = orc.fixed_prob_rows(5, range(n), n, K)
  for i, (r, f) in enumerate(zip(rows, full)):
    assert np.array_equal(r, f[f != i])
