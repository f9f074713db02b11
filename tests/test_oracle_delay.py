"""The oracle's network with synaptic delays (VarDelay in its rotating form,
brainpy/_src/delay.py:334-373) on the CPU: no delay reproduces the plain runner, a one-step
delay equals no delay from a silent start, a run split in two equals one run, and a delay
moves the propagated spikes later."""
import numpy as np


def _net(n=400, ne=320, k=20, seed=0):
  rng = np.random.default_rng(seed)
  ind = np.concatenate([rng.choice(n, k, replace=False) for _ in range(n)]).astype(np.int32)
  ptr = (np.arange(n + 1) * k).astype(np.int64)
  e_end = int(ptr[ne])
  return (ptr[: ne + 1].astype(np.int32), np.ascontiguousarray(ind[:e_end]),
          (ptr[ne:] - e_end).astype(np.int32), np.ascontiguousarray(ind[e_end:]))


def _state(n, seed=1):
  return {"V": np.random.default_rng(seed).normal(-55, 5, n).astype(np.float32), "ge": np.zeros(n, np.float32),
          "gi": np.zeros(n, np.float32), "t_last": np.full(n, -1e7, np.float32), "spike": np.zeros(n, np.uint8)}


def _run(orc, st, steps, de, di, step0=0, n=400, ne=320):
  p = orc.lif_params()
  ep, ei, ip, ii = _net(n, ne)
  return orc.coba_net_run_delayed(p, n, ne, ep, ei, np.float32(1.5), ip, ii, np.float32(6.7), st, step0, steps,
                                  np.float32(0.1), de, di)


def test_no_delay_is_the_plain_runner(orc):
  a, b = _state(400), _state(400)
  ca = _run(orc, a, 300, 0, 0)
  ep, ei, ip, ii = _net()
  cb, _ = orc.coba_net_run(orc.lif_params(), 400, 320, ep, ei, np.float32(1.5), ip, ii, np.float32(6.7), b, 0, 300,
                           np.float32(0.1))
  np.testing.assert_array_equal(ca, cb)
  for k in ("V", "ge", "gi", "t_last", "spike"):
    np.testing.assert_array_equal(a[k], b[k])
  assert ca.sum() > 100


def test_one_step_delay_equals_none_from_silence(orc):
  a, b = _state(400), _state(400)
  np.testing.assert_array_equal(_run(orc, a, 300, 1, 1), _run(orc, b, 300, 0, 0))
  np.testing.assert_array_equal(a["V"], b["V"])


def test_split_run_and_delay_effect(orc):
  a, b = _state(400), _state(400)
  whole = _run(orc, a, 300, 5, 3)
  first = _run(orc, b, 120, 5, 3)
  second = _run(orc, b, 180, 5, 3, step0=120)
  np.testing.assert_array_equal(whole, np.concatenate([first, second]))
  np.testing.assert_array_equal(a["V"], b["V"])
  c = _state(400)
  assert not np.array_equal(whole, _run(orc, c, 300, 0, 0))
