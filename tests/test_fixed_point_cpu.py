"""The arithmetic of fixed-weight plans, on the CPU: the exponent k and threshold tau that
event.fix_point_params picks, the int32 headroom of a column's integer sum, the 5e-6 bound on
every weight at or above tau, and the 24-bit records (the fit test and the split into low 16
bits and a high byte that the device rebuilds by sign replication).  The device converts a
weight as rint(float32(w) * 2^k), round half to even; numpy's float32 rint does the same."""
import numpy as np
import pytest

from brainpy_gb300.math.event import fix_fits_24, fix_point_params

LIM = 2.0 ** 31 - 2.0 ** 24


@pytest.mark.parametrize("bound", [1e-25, 1e-6, 0.37, 1.0, 555.7, 2.0 ** 20 + 3, 1e9])
def test_k_is_the_largest_safe_exponent(bound):
  k, tau = fix_point_params(bound)
  assert 0 <= k <= 100
  if 0 < k < 100:
    assert bound * 2.0 ** k <= LIM < bound * 2.0 ** (k + 1)
  assert tau == 2.0 ** -(k + 1) / 5e-6


def test_all_zero_matrix():
  assert fix_point_params(0.0)[0] == 30


def _weights(law, rng, shape):
  if law == "normal_0.5_0.1":
    return rng.normal(0.5, 0.1, shape)
  if law == "normal_0_1":
    return rng.normal(0.0, 1.0, shape)
  return rng.choice([-1.0, 1.0], shape) * 10.0 ** rng.uniform(-9, 3, shape)  # twelve decades


@pytest.mark.parametrize("law", ["normal_0.5_0.1", "normal_0_1", "wide"])
def test_weights_at_or_above_tau_within_5e_6(law):
  rng = np.random.default_rng(7)
  w = _weights(law, rng, (300, 1000)).astype(np.float32)  # 300 columns of 1000 inputs
  bound = float(np.abs(w.astype(np.float64)).sum(1).max())
  k, tau = fix_point_params(bound)
  q = np.rint(w * np.float32(2.0 ** k)).astype(np.int64)
  big = np.abs(w) >= tau
  err = np.abs(q * 2.0 ** -k - w.astype(np.float64))
  assert np.all(err[big] <= 5e-6 * np.abs(w[big]))
  assert np.abs(q).sum(1).max() < 2 ** 31  # no column's integer sum can overflow
  if fix_fits_24(float(np.abs(w).max()), k):
    assert np.all((q >= -(2 ** 23)) & (q < 2 ** 23))


def test_24_bit_fit_at_the_benchmarked_law():
  """N(0.5, 0.1) weights at fan-in ~1000 (largest column sum ~560): 24 bits with room to spare;
  N(0, 1) weights at the same fan-in reach past 2^23."""
  rng = np.random.default_rng(8)
  for law, fits in (("normal_0.5_0.1", True), ("normal_0_1", False)):
    w = _weights(law, rng, (2000, 1000)).astype(np.float32)
    k, _ = fix_point_params(float(np.abs(w.astype(np.float64)).sum(1).max()))
    assert fix_fits_24(float(np.abs(w).max()), k) == fits


def test_low_half_and_high_byte_rebuild_every_24_bit_value():
  """The 40-byte records store q & 0xFFFF and (q >> 16) & 0xFF; the device rebuilds q by
  replicating the high byte's sign over the top byte (a byte permute): the round trip is
  exact over [-2^23, 2^23)."""
  q = np.concatenate([np.arange(-(2 ** 23), -(2 ** 23) + 70000), np.arange(-70000, 70000),
                      np.arange(2 ** 23 - 70000, 2 ** 23),
                      np.random.default_rng(9).integers(-(2 ** 23), 2 ** 23, 200000)]).astype(np.int32)
  u = q.view(np.uint32)
  lo = (u & 0xFFFF).astype(np.int64)
  hi = ((u >> 16) & 0xFF).astype(np.uint8).view(np.int8).astype(np.int64)
  np.testing.assert_array_equal(hi * 65536 + lo, q.astype(np.int64))
