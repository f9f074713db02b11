"""jitconn operators on the GPU.

* connectivity and weights of every golden configuration (generated from the reference's
  own Taichi kernels) reproduced bit for bit by the kernels (normal weights: CUDA logf/sinf
  vs the fixtures' numpy float32 within a few ulp);
* y = M v against the FP64 oracle within 1e-5 scaled by sum|terms|, for every kind, vector
  type, outdim_parallel and algorithm variant;
* the reference test-suite properties: same seed -> same result, (shape, transpose) equals
  (reversed shape, not transpose);
* full size (4M x 4M, p = 2.5e-4): exact linearity in the event set."""
import ctypes

import numpy as np
import pytest
import torch

from golden_util import jitconn_keys, load, scaled_err

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def jc(bplib):
  from brainpy_gb300.math import jitconn
  return jitconn


def _dense(kind, p0, p1, clen, seed, nr, nc, odp, variant):
  from brainpy_gb300 import _lib
  d = torch.empty((nr, nc), dtype=torch.float32, device="cuda")
  st = _lib.lib().bp_jitconn_dense({"homo": 0, "uniform": 1, "normal": 2}[kind], p0, p1, clen, seed, nr, nc, int(odp),
                                   0 if variant == "gpu" else 1, ctypes.c_void_p(d.data_ptr()),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
  assert st == 0, _lib.lib().bp_last_error()
  return d.cpu().numpy()


def test_connectivity_matches_golden(jc):
  g = load("jitconn")
  n_checked = 0
  for key in jitconn_keys(g):
    kind, _, _, odp, dev, ev = key.split("|")
    if ev != "ev0":  # the dense-vector kernels expose every weight; event kernels share the matrix
      continue
    nr, nc, clen, seed = (int(x) for x in g[key + "|meta"])
    p0, p1 = (float(x) for x in g[key + "|par"])
    d = _dense(kind, p0, p1, clen, seed, nr, nc, odp == "odp1", dev)
    rows, cols, w = g[key + "|rows"], g[key + "|cols"], g[key + "|w"]
    expect = np.zeros((nr, nc), np.float32)
    expect[rows, cols] = w
    assert np.array_equal(d != 0, expect != 0), key
    if kind == "normal":
      np.testing.assert_allclose(d, expect, rtol=4e-6, atol=4e-6, err_msg=key)
    else:
      np.testing.assert_array_equal(d, expect, err_msg=key)
    # the event kernels of the same configuration walk the same connections
    ek = key[:-3] + "ev1"
    er, ec = g[ek + "|rows"], g[ek + "|cols"]
    assert set(zip(er.tolist(), ec.tolist())) == set(zip(rows.tolist(), cols.tolist())), ek
    n_checked += 1
  assert n_checked == 168


KINDS = [("homo", 0.7, 0.0), ("uniform", -0.5, 1.5), ("normal", 0.2, 1.1)]


@pytest.mark.parametrize("kind,p0,p1", KINDS)
@pytest.mark.parametrize("variant", ["gpu", "cpu"])
@pytest.mark.parametrize("shape,prob", [((200, 300), 0.1), ((3000, 2500), 0.01), ((700, 20000), 0.002)])
def test_mv_against_oracle(jc, orc, kind, p0, p1, variant, shape, prob):
  rng = np.random.default_rng(hash((kind, variant, shape)) & 0xFFFF)
  seed = 1234
  for transpose in (False, True):
    n_in = shape[0] if transpose else shape[1]
    n_out = shape[1] if transpose else shape[0]
    for odp in (True, False):
      ev = rng.random(n_in) < 0.1
      evf = np.where(rng.random(n_in) < 0.5, rng.normal(size=n_in), 0.0).astype(np.float32)
      vec = rng.normal(size=n_in).astype(np.float32)
      clen = jc.conn_len(prob)
      for vk, v, fn in ((0, ev, "event"), (1, evf, "event"), (2, vec, "mv")):
        args = (p0,) if kind == "homo" else (p0, p1)
        op = getattr(jc, f"{'event_' if fn == 'event' else ''}mv_prob_{kind}")
        y = op(torch.as_tensor(v, device="cuda"), *args, prob, seed, shape=shape, transpose=transpose,
               outdim_parallel=odp, variant=variant).cpu().numpy()
        y64, a64 = orc.jitconn_mv(kind, v, n_out, p0, p1, clen, seed, odp, variant, vec_kind=vk)
        assert y.shape == (n_out,)
        assert scaled_err(y, y64, a64) < TOL, (kind, variant, shape, transpose, odp, vk)


def test_reference_test_properties(jc):
  """test_event_matvec_taichi.py:36-81: determinism and (shape, T) == (shape[::-1], not T)."""
  rng = np.random.default_rng(0)
  for shape in [(100, 200), (10, 1000), (2, 1000), (1000, 10), (1000, 2)]:
    for prob in (0.01, 0.1, 0.5):
      for transpose in (True, False):
        for odp in (True, False):
          events = torch.as_tensor(rng.random(shape[0] if transpose else shape[1]) < 0.1, device="cuda")
          r1 = jc.event_mv_prob_homo_taichi(events, 1.0, prob, 1234, shape=shape, transpose=transpose,
                                            outdim_parallel=odp)
          r2 = jc.event_mv_prob_homo_taichi(events, 1.0, prob, 1234, shape=shape, transpose=transpose,
                                            outdim_parallel=odp)
          r3 = jc.event_mv_prob_homo_taichi(events, 1.0, prob, 1234, shape=(shape[1], shape[0]),
                                            transpose=not transpose, outdim_parallel=odp)
          assert torch.equal(r1, r2) and torch.equal(r1, r3)


def test_errors(jc):
  v = torch.ones(10, device="cuda")
  with pytest.raises(ValueError, match="Shape mismatch"):
    jc.mv_prob_homo(v, 1.0, 0.1, 1, shape=(5, 11))
  with pytest.raises(ValueError, match="outdim_parallel"):
    jc.mv_prob_homo(v, 1.0, 0.1, 1, shape=(5, 10), outdim_parallel=1)
  with pytest.raises(TypeError):
    jc.event_mv_prob_homo(torch.ones(10, dtype=torch.int32, device="cuda"), 1.0, 0.1, 1, shape=(5, 10))


def test_full_size_linearity(jc):
  """4M x 4M just-in-time matrix, fan-in 1000 (p = 2.5e-4, conn_len 7999), homogeneous weight 1:
  per-row results are exact small integers, so event-set linearity holds bit for bit."""
  from brainpy_gb300.connect import bernoulli_events
  n = 4_000_000
  p = 1000 / 4e6
  assert jc.conn_len(p) == 7999
  ev = bernoulli_events(n, 0.02, seed=5)
  y = jc.event_mv_prob_homo(ev, 1.0, p, 42, shape=(n, n))
  assert torch.equal(y, torch.round(y))
  half = torch.zeros_like(ev)
  half[: n // 2] = ev[: n // 2]
  y1 = jc.event_mv_prob_homo(half, 1.0, p, 42, shape=(n, n))
  y2 = jc.event_mv_prob_homo(ev & ~half, 1.0, p, 42, shape=(n, n))
  assert torch.equal(y1 + y2, y)
  # mean in-degree from active inputs ~ 0.02 * fan-in, reduced by the stripe quirk (no
  # column at step*k - 1 and none beyond 32*step - 1)
  assert 15.0 < float(y.double().mean()) < 21.0


@pytest.mark.parametrize("odp", [True, False])
def test_full_size_against_oracle(jc, orc, odp):
  """4M x 4M just-in-time matrix, fan-in 1000, 2 % bool events, seed 42, element-wise against
  the oracle's generation of the same streams.  Pull form (outdim_parallel): 300 sampled output
  rows, each regenerated from its own stream.  Push form: every output row (the oracle walks
  the active inputs' streams only).  Weight 1: exact integer counts, compared bit for bit;
  weight 0.6: within 1e-5 scaled by the sum of the terms."""
  from brainpy_gb300.connect import bernoulli_events
  n = 4_000_000
  p = 1000 / 4e6
  clen = jc.conn_len(p)
  ev = bernoulli_events(n, 0.02, seed=5)
  ev_h = ev.cpu().numpy()
  rng = np.random.default_rng(9)
  rows = np.unique(np.concatenate([rng.integers(0, n, 296), [0, 1, n - 2, n - 1]]))
  for w in (1.0, 0.6):
    y = jc.event_mv_prob_homo(ev, w, p, 42, shape=(n, n), outdim_parallel=odp).cpu().numpy()
    if odp:
      y64, a64 = orc.jitconn_mv_rows("homo", ev_h, n, w, 0.0, clen, 42, rows)
      y = y[rows]
    else:
      y64, a64 = orc.jitconn_mv("homo", ev_h, n, w, 0.0, clen, 42, False)
    if w == 1.0:
      np.testing.assert_array_equal(y, y64.astype(np.float32))
      assert y64.sum() > 0
    else:
      assert scaled_err(y, y64, a64) < TOL
