"""Differentiation rules of the propagation operators on the GPU against the oracle.

Reverse mode (torch.autograd.grad) and forward mode (torch.autograd.forward_ad) of
event.csrmv, sparse.csrmv and the jitconn operators, with the reference's rules
(brainpy/_src/math/event/_csr_matvec.py:521-551, sparse/_csr_mv.py:211-240,
jitconn/_matvec_taichi.py:138-171).  Bars: the per-entry weight cotangent is bit-exact
(one float32 product per entry); sums are within 1e-5 of FP64, scaled by the sum of |terms|."""
import numpy as np
import pytest
import torch
from torch.autograd import forward_ad as fwad

from golden_util import scaled_err

pytestmark = pytest.mark.gpu
TOL = 1e-5
DEV = torch.device("cuda")


def _csr(rng, m, n, kmax):
  lens = rng.integers(0, kmax, m)
  lens[::5] = 0
  ind = np.concatenate([rng.choice(n, l, replace=False) for l in lens]).astype(np.int32)
  ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
  return ind, ptr


def _t(x, **kw):
  return torch.as_tensor(x, device=DEV, **kw)


def _dot_tol(a, b):
  """FP64 dot and its error scale."""
  return float(np.dot(a, b)), float(np.dot(np.abs(a), np.abs(b)))


CASES = [(300, 500, 40), (40000, 40000, 60)]  # plain CSR kernels; the planned (tiled) path


@pytest.mark.parametrize("m,n,kmax", CASES)
@pytest.mark.parametrize("transpose", [True, False])
@pytest.mark.parametrize("heter", [False, True])
@pytest.mark.parametrize("evkind", ["bool", "float"])
def test_event_csrmv_reverse(bplib, orc, m, n, kmax, transpose, heter, evkind):
  from brainpy_gb300.math import event
  rng = np.random.default_rng(m + 7 * transpose + 3 * heter)
  ind, ptr = _csr(rng, m, n, kmax)
  nin, nout = (m, n) if transpose else (n, m)
  data = rng.normal(size=ind.size).astype(np.float32) if heter else np.array([0.6], np.float32)
  mask = rng.random(nin) < 0.1
  ev = mask if evkind == "bool" else (rng.normal(size=nin) * mask).astype(np.float32)
  ct = rng.normal(size=nout).astype(np.float32)
  d = _t(data).requires_grad_(True)
  e = _t(ev)
  if evkind == "float":
    e.requires_grad_(True)
  y = event.csrmv(d, _t(ind), _t(ptr), e, shape=(m, n), transpose=transpose)
  r = orc.event_csrmv(data, ind, ptr, ev, (m, n), transpose)
  assert scaled_err(y.detach().cpu().numpy(), r["out64"], r["abs64"]) < TOL
  grads = torch.autograd.grad(y, [d, e] if evkind == "float" else [d], _t(ct))
  gd = grads[0].cpu().numpy()
  if heter:
    rows = np.repeat(np.arange(m), np.diff(ptr))
    evf = ev.astype(np.float32)
    want = evf[rows] * ct[ind] if transpose else evf[ind] * ct[rows]
    np.testing.assert_array_equal(gd, want.astype(np.float32))
  else:
    unit = orc.event_csrmv(np.float32(1.0), ind, ptr, ev, (m, n), transpose)["out64"]
    v, s = _dot_tol(ct.astype(np.float64), unit)
    assert gd.shape == (1,) and abs(gd[0] - v) <= TOL * max(s, 1.0)
  if evkind == "float":
    ge = grads[1].cpu().numpy()
    rr = orc.csrmv(data, ind, ptr, ct, (m, n), not transpose)
    assert scaled_err(ge, rr["out64"], rr["abs64"]) < TOL


@pytest.mark.parametrize("m,n,kmax", CASES)
@pytest.mark.parametrize("transpose", [True, False])
@pytest.mark.parametrize("heter", [False, True])
def test_event_csrmv_forward_mode(bplib, orc, m, n, kmax, transpose, heter):
  from brainpy_gb300.math import event
  rng = np.random.default_rng(11 + m)
  ind, ptr = _csr(rng, m, n, kmax)
  nin = m if transpose else n
  data = rng.normal(size=ind.size).astype(np.float32) if heter else np.array([0.6], np.float32)
  ddata = rng.normal(size=data.size).astype(np.float32)
  ev = (rng.normal(size=nin) * (rng.random(nin) < 0.1)).astype(np.float32)
  dev_ = rng.normal(size=nin).astype(np.float32)
  with fwad.dual_level():
    d = fwad.make_dual(_t(data), _t(ddata))
    e = fwad.make_dual(_t(ev), _t(dev_))
    y = event.csrmv(d, _t(ind), _t(ptr), e, shape=(m, n), transpose=transpose)
    tan = fwad.unpack_dual(y).tangent.cpu().numpy()
  a = orc.event_csrmv(ddata, ind, ptr, ev, (m, n), transpose)
  b = orc.csrmv(data, ind, ptr, dev_, (m, n), transpose)
  assert scaled_err(tan, a["out64"] + b["out64"], a["abs64"] + b["abs64"]) < TOL


@pytest.mark.parametrize("m,n,kmax", CASES)
@pytest.mark.parametrize("transpose", [True, False])
@pytest.mark.parametrize("heter", [False, True])
def test_sparse_csrmv_reverse_and_forward(bplib, orc, m, n, kmax, transpose, heter):
  from brainpy_gb300.math import sparse
  rng = np.random.default_rng(5 + m)
  ind, ptr = _csr(rng, m, n, kmax)
  nin, nout = (m, n) if transpose else (n, m)
  data = rng.normal(size=ind.size).astype(np.float32) if heter else np.array([-1.3], np.float32)
  vec = (rng.normal(size=nin) * (rng.random(nin) < 0.3)).astype(np.float32)
  ct = rng.normal(size=nout).astype(np.float32)
  d = _t(data).requires_grad_(True)
  v = _t(vec).requires_grad_(True)
  y = sparse.csrmv(d, _t(ind), _t(ptr), v, shape=(m, n), transpose=transpose)
  gd, gv = torch.autograd.grad(y, [d, v], _t(ct))
  gd, gv = gd.cpu().numpy(), gv.cpu().numpy()
  if heter:
    rows = np.repeat(np.arange(m), np.diff(ptr))
    want = vec[rows] * ct[ind] if transpose else vec[ind] * ct[rows]
    np.testing.assert_array_equal(gd, want.astype(np.float32))
  else:
    unit = orc.csrmv(np.float32(1.0), ind, ptr, vec, (m, n), transpose)["out64"]
    val, s = _dot_tol(ct.astype(np.float64), unit)
    assert abs(gd[0] - val) <= TOL * max(s, 1.0)
  rr = orc.csrmv(data, ind, ptr, ct, (m, n), not transpose)
  assert scaled_err(gv, rr["out64"], rr["abs64"]) < TOL
  ddata = rng.normal(size=data.size).astype(np.float32)
  dvec = rng.normal(size=nin).astype(np.float32)
  with fwad.dual_level():
    y = sparse.csrmv(fwad.make_dual(_t(data), _t(ddata)), _t(ind), _t(ptr), fwad.make_dual(_t(vec), _t(dvec)),
                     shape=(m, n), transpose=transpose)
    tan = fwad.unpack_dual(y).tangent.cpu().numpy()
  a = orc.csrmv(ddata, ind, ptr, vec, (m, n), transpose)
  b = orc.csrmv(data, ind, ptr, dvec, (m, n), transpose)
  assert scaled_err(tan, a["out64"] + b["out64"], a["abs64"] + b["abs64"]) < TOL


def test_sampled_outer_edges(bplib):
  """Entries outside every row and out-of-range columns get 0; the rest one product each."""
  from brainpy_gb300.math import _grad
  ind = np.array([9, 1, 2, 7, 0, 3, 5, 4], np.int64)  # 7 is out of range for n = 6
  ptr = np.array([1, 3, 3, 6], np.int64)  # entry 0 before row 0, entries 6-7 after the last row
  x = np.array([2.0, -1.0, 0.5], np.float32)
  y = np.arange(1, 7, dtype=np.float32)
  out = _grad.sampled_outer(_t(x), _t(y), _t(ind), _t(ptr), 3, 6).cpu().numpy()
  want = np.array([0, 2 * y[1], 2 * y[2], 0, 0.5 * y[0], 0.5 * y[3], 0, 0], np.float32)  # column 7 >= n: 0
  np.testing.assert_array_equal(out, want)


JC_SHAPES = [((300, 200), 0.05), ((64, 1000), 0.1)]


@pytest.mark.parametrize("kind", ["homo", "uniform", "normal"])
@pytest.mark.parametrize("event", [False, True])
@pytest.mark.parametrize("transpose", [False, True])
@pytest.mark.parametrize("outdim_parallel", [True, False])
@pytest.mark.parametrize("shape,prob", JC_SHAPES)
@pytest.mark.parametrize("variant", ["gpu", "cpu"])
def test_jitconn_reverse(bplib, orc, kind, event, transpose, outdim_parallel, shape, prob, variant):
  from brainpy_gb300.math import jitconn
  rng = np.random.default_rng(3)
  nin, nout = (shape[0], shape[1]) if transpose else (shape[1], shape[0])
  vec = (rng.normal(size=nin) * (rng.random(nin) < 0.4)).astype(np.float32)
  ct = rng.normal(size=nout).astype(np.float32)
  name = ("event_" if event else "") + f"mv_prob_{kind}"
  op = getattr(jitconn, name)
  v = _t(vec).requires_grad_(True)
  seed = 1234
  kw = dict(shape=shape, transpose=transpose, outdim_parallel=outdim_parallel, variant=variant)
  clen = jitconn.conn_len(prob)
  if kind == "homo":
    w = _t(np.array([0.8], np.float32)).requires_grad_(True)
    y = op(v, w, prob, seed, **kw)
    gv, gw = torch.autograd.grad(y, [v, w], _t(ct))
    p0, p1 = 0.8, 0.0
  else:
    p0, p1 = (-0.5, 1.5) if kind == "uniform" else (0.2, 0.9)
    y = op(v, p0, p1, prob, seed, **kw)
    (gv,) = torch.autograd.grad(y, [v], _t(ct))
  vk = 1 if event else 2
  y64, a64 = orc.jitconn_mv(kind, vec, nout, p0, p1, clen, seed, outdim_parallel, variant, vec_kind=vk)
  assert scaled_err(y.detach().cpu().numpy(), y64, a64) < TOL
  # the rule: the non-event product of ct with transpose and outdim_parallel flipped
  g64, ga64 = orc.jitconn_mv(kind, ct, nin, p0, p1, clen, seed, not outdim_parallel, variant, vec_kind=2)
  assert scaled_err(gv.cpu().numpy(), g64, ga64) < TOL
  if variant == "cpu":
    # with the Taichi CPU connectivity the flipped call regenerates M^T exactly, so the rule
    # is the adjoint: <ct, M v> = <M^T ct, v>, M applied to the event indicator (!= 0) or
    # the dense vector.  (The GPU connectivity splits lanes by the owner count and does not
    # have this symmetry; the rule is the reference's all the same.)
    vin = (vec != 0).astype(np.float64) if event else vec.astype(np.float64)
    mv = orc.jitconn_mv(kind, vin.astype(np.float32), nout, p0, p1, clen, seed, outdim_parallel, variant,
                        vec_kind=2)[0]
    lhs, s1 = _dot_tol(ct.astype(np.float64), mv)
    rhs, s2 = _dot_tol(g64, vin)
    assert abs(lhs - rhs) <= 1e-9 * max(s1, s2, 1.0)
  if kind == "homo":
    unit, ua = orc.jitconn_mv(kind, vec, nout, 1.0, 0.0, clen, seed, outdim_parallel, variant, vec_kind=vk)
    val, s = _dot_tol(ct.astype(np.float64), unit)
    assert abs(float(gw.cpu()[0]) - val) <= TOL * max(s, 1.0)


@pytest.mark.parametrize("kind", ["homo", "normal"])
@pytest.mark.parametrize("outdim_parallel", [True, False])
def test_jitconn_forward_mode(bplib, orc, kind, outdim_parallel):
  from brainpy_gb300.math import jitconn
  rng = np.random.default_rng(9)
  shape, prob, seed = (250, 400), 0.05, 77
  vec = rng.normal(size=400).astype(np.float32)
  dvec = rng.normal(size=400).astype(np.float32)
  clen = jitconn.conn_len(prob)
  with fwad.dual_level():
    v = fwad.make_dual(_t(vec), _t(dvec))
    if kind == "homo":
      w = fwad.make_dual(_t(np.array([0.5], np.float32)), _t(np.array([2.0], np.float32)))
      y = jitconn.mv_prob_homo(v, w, prob, seed, shape=shape, outdim_parallel=outdim_parallel)
      p0, p1 = 0.5, 0.0
    else:
      y = jitconn.mv_prob_normal(v, 0.1, 1.0, prob, seed, shape=shape, outdim_parallel=outdim_parallel)
      p0, p1 = 0.1, 1.0
    tan = fwad.unpack_dual(y).tangent.cpu().numpy()
  t64, ta = orc.jitconn_mv(kind, dvec, 250, p0, p1, clen, seed, outdim_parallel)
  if kind == "homo":
    u64, ua = orc.jitconn_mv(kind, vec, 250, 1.0, 0.0, clen, seed, outdim_parallel)
    t64, ta = t64 + 2.0 * u64, ta + 2.0 * ua
  assert scaled_err(tan, t64, ta) < TOL


def test_layer_weight_training_step(bplib, orc):
  """EventCSRLinear with a trainable heterogeneous weight: one SGD step moves exactly the
  entries of active rows, by lr * ct[col]."""
  from brainpy_gb300 import dnn
  rng = np.random.default_rng(4)
  m, n = 200, 300
  ind, ptr = _csr(rng, m, n, 30)
  w = _t(rng.normal(size=ind.size).astype(np.float32)).requires_grad_(True)
  layer = dnn.EventCSRLinear((_t(ind), _t(ptr)), w, shape=(m, n))
  ev = rng.random(m) < 0.2
  ct = rng.normal(size=n).astype(np.float32)
  y = layer(_t(ev))
  (g,) = torch.autograd.grad(y, [w], _t(ct))
  rows = np.repeat(np.arange(m), np.diff(ptr))
  np.testing.assert_array_equal(g.cpu().numpy(), (ev[rows].astype(np.float32) * ct[ind]).astype(np.float32))
