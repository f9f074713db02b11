"""The projection layers (brainpy/_src/dnn/linear.py) call the operators exactly as the
reference does: same shapes, transpose and outdim_parallel = not atomic."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _close(a, b):
  """float32 sums accumulated by shared-memory atomics: equal up to summation order"""
  a, b = a.double(), b.double()
  return bool(((a - b).abs() <= 1e-5 * torch.clamp(b.abs(), min=1.0)).all())


@pytest.fixture(scope="module")
def mods(bplib):
  from brainpy_gb300 import dnn
  from brainpy_gb300.math import event, jitconn, sparse
  return dnn, event, jitconn, sparse


class _Conn:
  """A BrainPy-style connector: require('csr'), pre_num, post_num."""

  def __init__(self, indices, indptr, pre, post):
    self.i, self.p, self.pre_num, self.post_num = indices, indptr, pre, post

  def require(self, what):
    assert what == "csr"
    return self.i, self.p


def test_csr_layers(mods):
  dnn, event, jitconn, sparse = mods
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr
  pre, post = 3000, 2000
  ind, ptr = fixed_prob_csr(pre, post, 40, seed=3)
  conn = _Conn(ind, ptr, pre, post)
  spk = bernoulli_events(pre, 0.1, seed=4)
  lay = dnn.EventCSRLinear(conn, 0.5)
  assert torch.equal(lay(spk), event.csrmv(0.5, ind, ptr, spk, shape=(pre, post), transpose=True))
  w = torch.rand(ind.numel(), device="cuda")
  lay = dnn.EventCSRLinear((ind, ptr), w, shape=(pre, post))
  batch = torch.stack([spk, bernoulli_events(pre, 0.3, seed=5)])
  y = lay(batch)
  assert y.shape == (2, post)
  assert _close(y[1], event.csrmv(w, ind, ptr, batch[1], shape=(pre, post), transpose=True))
  assert _close(y[0], event.csrmv(w, ind, ptr, batch[0], shape=(pre, post), transpose=True))
  x = torch.randn(pre, device="cuda")
  lay = dnn.CSRLinear(conn, w)
  assert _close(lay(x), sparse.csrmv(w, ind, ptr, x, shape=(pre, post), transpose=True))
  lay = dnn.CSRLinear(conn, w, transpose=False)
  xr = torch.randn(post, device="cuda")
  assert _close(lay(xr), sparse.csrmv(w, ind, ptr, xr, shape=(pre, post), transpose=False))
  with pytest.raises(ValueError):
    dnn.CSRLinear((ind, ptr), w)  # shape missing
  with pytest.raises(ValueError):
    dnn.EventCSRLinear(conn, torch.ones(5, device="cuda"))


@pytest.mark.parametrize("atomic", [False, True])
def test_jit_layers(mods, atomic):
  dnn, event, jitconn, sparse = mods
  from brainpy_gb300.connect import bernoulli_events
  n_in, n_out, p = 5000, 3000, 0.02
  spk = bernoulli_events(n_in, 0.05, seed=6)
  x = torch.randn(n_in, device="cuda")
  cases = [
      (dnn.EventJitFPHomoLinear(n_in, n_out, p, 0.7, seed=11, atomic=atomic), jitconn.event_mv_prob_homo, (0.7,), spk),
      (dnn.EventJitFPUniformLinear(n_in, n_out, p, 0.1, 0.9, seed=12, atomic=atomic), jitconn.event_mv_prob_uniform,
       (0.1, 0.9), spk),
      (dnn.EventJitFPNormalLinear(n_in, n_out, p, 0.0, 1.0, seed=13, atomic=atomic), jitconn.event_mv_prob_normal,
       (0.0, 1.0), spk),
      (dnn.JitFPHomoLinear(n_in, n_out, p, 0.7, seed=14, atomic=atomic), jitconn.mv_prob_homo, (0.7,), x),
      (dnn.JitFPUniformLinear(n_in, n_out, p, 0.1, 0.9, seed=15, atomic=atomic), jitconn.mv_prob_uniform, (0.1, 0.9), x),
      (dnn.JitFPNormalLinear(n_in, n_out, p, 0.0, 1.0, seed=16, atomic=atomic), jitconn.mv_prob_normal, (0.0, 1.0), x),
  ]
  for lay, op, w, v in cases:
    y = lay(v)
    ref = op(v, *w, p, lay.seed, shape=(n_out, n_in), outdim_parallel=not atomic)
    assert y.shape == (n_out,)
    if atomic:  # push form: float atomics, summation order varies
      assert _close(y, ref)
    else:
      np.testing.assert_array_equal(y.cpu().numpy(), ref.cpu().numpy())
  lay = dnn.EventJitFPHomoLinear(n_in, n_out, p, 0.7, atomic=atomic)
  assert 0 <= lay.seed < 1000000
