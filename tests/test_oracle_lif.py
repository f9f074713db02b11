"""Known-answer tests pinning the oracle's LIF / Expon / COBA step.

The exponential-Euler rule of the reference (integrators/ode/exponential.py:354-362)
is exact for linear ODEs, which gives closed-form answers:
  Expon:       g' = g * exp(-dt / tau)
  LIF (g = 0): V' = V_inf + (V - V_inf) * exp(-dt / tau),  V_inf = V_rest + R * I
  LifRefLTC with constant conductances:
               V' = V_inf + (V - V_inf) * exp(-dt * (1 + R*(ge+gi)) / tau),
               V_inf = (V_rest + R*(I + ge*Ee + gi*Ei)) / (1 + R*(ge+gi))
"""
import ctypes
import math

import numpy as np


def _state(n, V0):
  return dict(V=np.full(n, V0, np.float32), ge=np.zeros(n, np.float32), gi=np.zeros(n, np.float32),
              t_last=np.full(n, -1e7, np.float32), spike=np.zeros(n, np.uint8))


def _step(orc, p, s, dge=None, dgi=None, i=0, dt=0.1, precise=False):
  n = s["V"].shape[0]
  dge = np.zeros(n, np.float32) if dge is None else dge.astype(np.float32)
  dgi = np.zeros(n, np.float32) if dgi is None else dgi.astype(np.float32)
  orc.lif_step(p, s["V"], s["ge"], s["gi"], s["t_last"], s["spike"], dge, dgi, i, dt, precise)


def test_free_membrane_closed_form(orc):
  p = orc.lif_params(input=20.0, ltc=True)
  V0 = -55.0
  for precise in (False, True):
    s = _state(1, V0)
    _step(orc, p, s, precise=precise)
    v_inf = -60.0 + 20.0
    exact = v_inf + (V0 - v_inf) * math.exp(-0.1 / 20.0)
    assert abs(float(s["V"][0]) - exact) < (2e-5 if not precise else 1e-5)


def test_expon_closed_form(orc):
  p = orc.lif_params(input=0.0)
  s = _state(2, -70.0)
  _step(orc, p, s, dge=np.array([2.0, 0.0]), dgi=np.array([0.0, 3.0]))
  assert abs(float(s["ge"][0]) - 2.0 * math.exp(-0.1 / 5.0)) < 2e-6
  assert abs(float(s["gi"][1]) - 3.0 * math.exp(-0.1 / 10.0)) < 2e-6


def test_ltc_constant_conductance_closed_form(orc):
  p = orc.lif_params(input=20.0, ltc=True, tau_e=1e30, tau_i=1e30)  # conductances frozen
  s = _state(1, -58.0)
  ge, gi = 0.4, 0.25
  s["ge"][:] = ge
  s["gi"][:] = gi
  _step(orc, p, s, precise=True)
  lam = (1 + ge + gi) / 20.0
  v_inf = (-60.0 + (20.0 + ge * 0.0 + gi * -80.0)) / (1 + ge + gi)
  exact = v_inf + (-58.0 - v_inf) * math.exp(-0.1 * lam)
  assert abs(float(s["V"][0]) - exact) < 1e-5


def test_refractory_threshold_reset(orc):
  p = orc.lif_params(input=2000.0)  # drives V over threshold in one step
  s = _state(1, -55.0)
  _step(orc, p, s, i=10)
  assert s["spike"][0] == 1 and s["V"][0] == np.float32(-60.0)
  assert s["t_last"][0] == np.float32(10) * np.float32(0.1)
  v_before = float(s["V"][0])
  _step(orc, p, s, i=11)  # t - t_last = 0.1 <= 5 -> refractory, V held
  assert s["spike"][0] == 0 and float(s["V"][0]) == v_before


def test_f32_mode_tracks_f64_mode(orc):
  rng = np.random.default_rng(3)
  n = 512
  p = orc.lif_params()
  a = _state(n, 0.0)
  a["V"][:] = rng.normal(-55, 5, n).astype(np.float32)
  b = {k: v.copy() for k, v in a.items()}
  diverged = np.zeros(n, bool)
  for i in range(100):
    dge = (rng.random(n) < 0.05).astype(np.float32) * 0.6
    dgi = (rng.random(n) < 0.02).astype(np.float32) * 6.7
    _step(orc, p, a, dge, dgi, i=i)
    _step(orc, p, b, dge, dgi, i=i, precise=True)
    diverged |= a["spike"] != b["spike"]
  # a threshold crossing decided differently by float32 rounding separates a neuron's
  # trajectory for good; all others must agree closely
  assert diverged.mean() < 0.01
  assert np.max(np.abs(a["V"][~diverged] - b["V"][~diverged])) < 1e-3


def test_deterministic_exp_accuracy(orc):
  """bp_expf (shared by the oracle and the kernels) against the C library's expf: within 1 ulp."""
  libm = ctypes.CDLL("libm.so.6")
  libm.expf.restype = ctypes.c_float
  libm.expf.argtypes = [ctypes.c_float]
  xs = np.concatenate([np.linspace(-0.2, 0.2, 4001), np.linspace(-87, 88, 4001),
                       -np.logspace(-8, 1, 500)]).astype(np.float32)
  worst = 0
  for x in xs:
    a = np.float32(orc.lib().orc_bp_expf(float(x)))
    b = np.float32(libm.expf(float(x)))
    ulp = np.spacing(np.abs(b))
    worst = max(worst, float(abs(np.float64(a) - np.float64(b)) / ulp))
  assert worst <= 1.0
  # exprel: series branch below 1e-5, quotient above
  assert orc.lib().orc_bp_exprel(0.0) == 1.0
  x = np.float32(-0.005)
  ref = math.expm1(float(x)) / float(x)
  assert abs(orc.lib().orc_bp_exprel(float(x)) - ref) < 3e-5
