"""The oracle's neuron / synapse consumer pinned to the reference's own code.

tests/golden/consumer.npz comes from tests/golden/make_golden.py, which executes the
reference's methods themselves (ast-extracted, run on numpy float32 with stand-ins for
bm.vector_grad / bm.exprel / share):
  LifLTC.derivative, LifRefLTC.update, LifRef.derivative / .update (dyn/neurons/lif.py),
  Expon.derivative / .update / .add_current (dyn/synapses/abstract_models.py),
  COBA.update (dyn/outs/outputs.py), the exponential-Euler integral
  (integrators/ode/exponential.py:338-364), _exprel (math/others.py), the input sums of
  mixin.py:427-469, and VarDelay.at / .retrieve / .update (delay.py:277-373),
stepped in the order of the E/I COBA example's projections (align_post.py:271-275).

Bars: membrane potentials within 1e-4 mV over the first 100 steps, spike counts per step
equal over those steps; the rotating delay's reads are the reference's."""
import numpy as np
import pytest

from golden_util import load


@pytest.fixture(scope="module")
def cons():
  return load("consumer")


def _net(orc, cons, ltc, d_e, d_i, steps, trace):
  n_exc, n_inh = (int(x) for x in cons["sizes"])
  n = n_exc + n_inh
  we, wi = (float(x) for x in cons["weights"])
  p = orc.lif_params(input=20.0, ltc=bool(ltc))
  st = dict(V=cons["V0"].copy(), ge=np.zeros(n, np.float32), gi=np.zeros(n, np.float32),
            t_last=np.full(n, -1e7, np.float32), spike=np.zeros(n, np.uint8))
  args = (p, n, n_exc, cons["ptr_e"], cons["ind_e"], we, cons["ptr_i"], cons["ind_i"], wi, st, 0, steps, 0.1)
  if d_e == 0 and d_i == 0:
    counts, tr = orc.coba_net_run(*args, trace_steps=trace)
    return counts, tr, st
  counts = orc.coba_net_run_delayed(*args, d_e, d_i)
  return counts, None, st


@pytest.mark.parametrize("tag", ["ltc", "lifref"])
def test_network_trajectory_matches_reference(orc, cons, tag):
  ltc, d_e, d_i = (int(x) for x in cons[f"{tag}|cfg"])
  counts, tr, _ = _net(orc, cons, ltc, d_e, d_i, 100, 100)
  want_V = cons[f"{tag}|V"]
  assert np.max(np.abs(tr - want_V)) < 1e-4
  np.testing.assert_array_equal(counts, cons[f"{tag}|counts"][:100])


@pytest.mark.parametrize("tag", ["ltc_d3_1", "ltc_d2_0"])
def test_delayed_network_matches_reference(orc, cons, tag):
  ltc, d_e, d_i = (int(x) for x in cons[f"{tag}|cfg"])
  counts, _, st = _net(orc, cons, ltc, d_e, d_i, 100, 0)
  assert np.max(np.abs(st["V"] - cons[f"{tag}|V"][99])) < 1e-4
  np.testing.assert_array_equal(counts, cons[f"{tag}|counts"][:100])


def test_rotating_delay_reads(cons):
  """VarDelay (rotation): at step i a delay of d steps reads what step i - d produced (nothing
  before the first d steps), for every ring length L >= d -- the rule the oracle's and the
  device's spike-history rings implement (slot T mod L written at step T, slot (T - d) mod L
  read)."""
  for key in [k for k in cons.files if k.startswith("delay|")]:
    _, L, d = key.split("|")
    L, d = int(L[1:]), int(d[1:])
    read = cons[key]
    want = np.array([i - d if i >= d else -1 for i in range(read.shape[0])])
    np.testing.assert_array_equal(read, want, err_msg=key)
