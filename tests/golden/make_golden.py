"""Generates the golden fixtures in this directory by executing the REFERENCE's
own kernel source code (BrainPy) in plain Python.

The reference's native stacks (Taichi, Numba, JAX, brainpylib) are not
installable here, so this script

* parses the reference files with ``ast`` and pulls out the kernel functions
  by name (the modules themselves cannot be imported: they import jax);
* runs the Taichi kernels against ``ti_emulator`` (integer types with C++
  promotion and 32-bit wrap, float32 arithmetic, serial loops);
* runs the Numba kernels as plain Python on numpy arrays (``njit`` becomes the
  identity, ``prange`` becomes ``range``; the float accumulator ``r = 0.`` is
  made float64, the type Numba infers for it);
* traces the just-in-time-connectivity kernels: the input vector hands out
  tracer objects and the output records every addition, which recovers the
  complete connection list (row, column, weight) in generation order.

Run from the repository root:  python tests/golden/make_golden.py
It reads the reference tree given by BRAINPY_REF (default /root/reference) and
writes tests/golden/*.npz.  The fixtures are committed; tests never need the
reference tree.
"""
import ast
import inspect
import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ti_emulator  # noqa: E402

REF = os.environ.get("BRAINPY_REF", "/root/reference")
MATH = os.path.join(REF, "brainpy", "_src", "math")


def load_functions(path, names, ns):
  """Exec the top-level function definitions `names` of `path` inside `ns`."""
  src = open(path).read()
  tree = ast.parse(src)
  wanted = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
  found = {n.name for n in wanted}
  missing = set(names) - found
  if missing:
    raise RuntimeError(f"{path}: missing {sorted(missing)}")
  mod = ast.Module(body=wanted, type_ignores=[])
  exec(compile(mod, path, "exec"), ns)
  return ns


class Float64Accumulators(ast.NodeTransformer):
  """`r = 0.` -> `r = np.float64(0.)`: Numba types that accumulator as float64."""

  def visit_Assign(self, node):
    if (len(node.targets) == 1 and isinstance(node.targets[0], ast.Name)
        and isinstance(node.value, ast.Constant) and isinstance(node.value.value, float)):
      node.value = ast.parse(f"np.float64({node.value.value!r})").body[0].value
    return node


def load_numba_functions(path, names, ns):
  src = open(path).read()
  tree = ast.parse(src)
  wanted = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
  if len(wanted) != len(names):
    raise RuntimeError(f"{path}: missing some of {names}")
  for n in wanted:
    n.decorator_list = []
  mod = Float64Accumulators().visit(ast.Module(body=wanted, type_ignores=[]))
  ast.fix_missing_locations(mod)
  exec(compile(mod, path, "exec"), ns)
  return ns


# --------------------------------------------------------------------------
# Taichi namespace: tifunc.py with the emulated taichi module
# --------------------------------------------------------------------------
ti = ti_emulator.make_module()
defaults = types.SimpleNamespace(ti_float=ti_emulator.f32, ti_int=ti_emulator.i32)
TI_NS = {"ti": ti, "defaults": defaults, "np": np}
load_functions(os.path.join(MATH, "tifunc.py"),
               ["lfsr88_key", "lfsr88_next_key", "lfsr88_normal", "lfsr88_randn",
                "lfsr88_random_integers", "lfsr88_randint", "lfsr88_uniform", "lfsr88_rand"], TI_NS)


class Arr:
  """ndarray argument of an emulated Taichi kernel."""

  def __init__(self, a):
    self.a = a
    self.shape = a.shape

  def __getitem__(self, i):
    v = self.a[int(i)]
    if self.a.dtype == np.uint32:
      return ti_emulator.u32(int(v))
    if self.a.dtype == np.int32:
      return ti_emulator.i32(int(v))
    if self.a.dtype == np.bool_:
      return bool(v)
    return v

  def __setitem__(self, i, v):
    self.a[int(i)] = v


# ---- tracing objects for connectivity extraction -------------------------
class Term:
  __array_ufunc__ = None

  def __init__(self, terms):
    self.terms = terms  # list of (col, w)

  def __radd__(self, o):
    if isinstance(o, (float, np.floating)) and float(o) == 0.0:
      return Term(list(self.terms))
    raise TypeError(o)

  def __add__(self, o):
    if isinstance(o, Term):
      return Term(self.terms + o.terms)
    if isinstance(o, Tracer):
      return Term(self.terms + [(o.col, np.float32(1.0))])
    raise TypeError(o)

  def __rmul__(self, w):
    return Term([(c, np.float32(w) * x) for c, x in self.terms])

  __mul__ = __rmul__


class Tracer:
  """Stands for vector[col]: true in every event test, records the column."""
  __array_ufunc__ = None

  def __init__(self, col):
    self.col = col

  def __bool__(self):
    return True

  def __ne__(self, o):
    return True

  def __gt__(self, o):
    return True

  def __mul__(self, w):
    return Term([(self.col, np.float32(w))])

  __rmul__ = __mul__

  def __radd__(self, o):
    if isinstance(o, (float, np.floating)) and float(o) == 0.0:
      return Term([(self.col, np.float32(1.0))])
    raise TypeError(o)


class TraceVec:
  def __init__(self, n):
    self.shape = (n,)
    self.last = None
    self.accessed = []

  def __getitem__(self, i):
    self.last = int(i)
    self.accessed.append(int(i))
    return Tracer(int(i))

  def drain(self):
    a, self.accessed = self.accessed, []
    return a


class Acc:
  def __init__(self, out, row):
    self.out, self.row = out, row

  def __add__(self, x):
    if isinstance(x, Term):
      for c, w in x.terms:
        self.out.log.append((self.row, c, np.float32(w)))
    elif isinstance(x, (float, np.floating)):
      # a bare float is one push-kernel connection onto the column tested last;
      # an exact 0.0 is the empty accumulator of a pull-kernel lane
      if float(x) != 0.0:
        assert self.out.vec.last is not None
        self.out.log.append((self.row, self.out.vec.last, np.float32(x)))
    else:
      raise TypeError(x)
    return self

  __iadd__ = __add__


class TraceOut:
  def __init__(self, n, vec):
    self.shape = (n,)
    self.vec = vec
    self.log = []

  def __getitem__(self, i):
    return Acc(self, int(i))

  def __setitem__(self, i, v):
    if isinstance(v, Acc):
      self.vec.drain()
      return
    if isinstance(v, Term):  # CPU pull kernels assign out[i_row] = r
      self.vec.drain()
      for c, w in v.terms:
        self.log.append((int(i), c, np.float32(w)))
      return
    if isinstance(v, (float, np.floating)):
      # CPU pull event kernels: `if events[c]: r += w` leaves a plain float; the
      # connections are the columns tested since the previous row, the
      # individual weights are not observable (recorded as NaN)
      for c in self.vec.drain():
        self.log.append((int(i), c, np.float32(np.nan)))
      return
    raise TypeError(v)


def taichi_clen(prob):
  """clen of the *_taichi front-ends: jnp.ceil(1 / conn_prob) * 2 - 1 with 1/p in
  Python double, ceil on float32 (_event_matvec_taichi.py:401-402)."""
  return int(math.ceil(np.float32(1.0 / prob))) * 2 - 1


def jitconn_kernel_names():
  names = []
  for kind in ("homo", "uniform", "normal"):
    for pre in ("_event_mv_prob_", "_mv_prob_"):
      for odp in ("outdim_parallel_", ""):
        for dev in ("gpu", "cpu"):
          if pre == "_event_mv_prob_":
            names.append(f"{pre}{kind}_{odp}bool_{dev}")
          else:
            names.append(f"{pre}{kind}_{odp}{dev}")
  return names


def gen_jitconn():
  ns = dict(TI_NS)
  names = jitconn_kernel_names()
  ev_names = [n for n in names if n.startswith("_event_")]
  mv_names = [n for n in names if not n.startswith("_event_")]
  load_functions(os.path.join(MATH, "jitconn", "_event_matvec_taichi.py"), ev_names, ns)
  load_functions(os.path.join(MATH, "jitconn", "_matvec_taichi.py"), mv_names, ns)
  out = {}
  shapes = [(100, 200), (2, 1000), (1000, 2), (300, 300), (64, 40)]
  probs = [0.01, 0.1, 0.5]
  seed = 1234
  params = {"homo": (1.5, None), "uniform": (-1.0, 2.0), "normal": (0.5, 1.2)}
  for kind, (p0, p1) in params.items():
    for (num_row, num_col) in shapes:
      for prob in probs:
        if (num_row, num_col) == (300, 300) and prob == 0.5:
          continue
        clen = taichi_clen(prob)
        for odp in (1, 0):
          for dev in ("gpu", "cpu"):
            for event in (1, 0):
              pre = "_event_mv_prob_" if event else "_mv_prob_"
              name = f"{pre}{kind}_{'outdim_parallel_' if odp else ''}{'bool_' if event else ''}{dev}"
              fn = ns[name]
              vec = TraceVec(num_col)
              o = TraceOut(num_row, vec)
              args = [vec]
              args.append(Arr(np.array([p0], np.float32)))
              if p1 is not None:
                args.append(Arr(np.array([p1], np.float32)))
              args += [Arr(np.array([clen], np.int32)), Arr(np.array([seed], np.uint32)), o]
              fn(*args)
              log = o.log
              rows = np.array([r for r, c, w in log], np.int32)
              cols = np.array([c for r, c, w in log], np.int32)
              ws = np.array([w for r, c, w in log], np.float32)
              key = f"{kind}|{num_row}x{num_col}|p{prob}|odp{odp}|{dev}|ev{event}"
              out[key + "|rows"] = rows
              out[key + "|cols"] = cols
              out[key + "|w"] = ws
              out[key + "|meta"] = np.array([num_row, num_col, clen, seed], np.int64)
              out[key + "|par"] = np.array([p0, p1 if p1 is not None else 0.0], np.float32)
  return out


def gen_lfsr():
  ns = TI_NS
  out = {}
  seeds = [0, 1, 42, 1234, 4294967280]
  for s in seeds:
    key = ns["lfsr88_key"](ti_emulator.u32(s))
    xs = []
    for _ in range(16):
      key, x = ns["lfsr88_randint"](key)
      xs.append(int(x))
    out[f"randint|{s}"] = np.array(xs, np.uint32)
    for (lo, hi) in [(1, 19), (0, 198), (1, 7999)]:
      key = ns["lfsr88_key"](ti_emulator.u32(s))
      ys = []
      for _ in range(16):
        key, y = ns["lfsr88_random_integers"](key, lo, ti_emulator.i32(hi))
        ys.append(int(y))
      out[f"random_integers|{s}|{lo}|{hi}"] = np.array(ys, np.int32)
    for (lo, hi) in [(0.0, 1.0), (-2.5, 3.5)]:
      key = ns["lfsr88_key"](ti_emulator.u32(s))
      ys = []
      for _ in range(16):
        key, y = ns["lfsr88_uniform"](key, np.float32(lo), np.float32(hi))
        ys.append(np.float32(y))
      out[f"uniform|{s}|{lo}|{hi}"] = np.array(ys, np.float32)
    for (mu, sd) in [(0.0, 1.0), (0.5, 0.1)]:
      key = ns["lfsr88_key"](ti_emulator.u32(s))
      ys = []
      for _ in range(16):
        key, y = ns["lfsr88_normal"](key, np.float32(mu), np.float32(sd))
        ys.append(np.float32(y))
      out[f"normal|{s}|{mu}|{sd}"] = np.array(ys, np.float32)
  return out


def fixed_prob_csr(rng, m, n, prob):
  """Fixed fan-out int(n*prob) distinct columns per row, unsorted (the shape of
  bp.conn.FixedProb(prob).require('pre2post'), random_conn.py:118-128)."""
  k = int(n * prob)
  indices = np.concatenate([rng.permutation(n)[:k] for _ in range(m)]).astype(np.int32) if k else np.zeros(0, np.int32)
  indptr = (np.arange(m + 1) * k).astype(np.int32)
  return indices, indptr


def gen_csr():
  ns = {"np": np, "numba": types.SimpleNamespace(prange=range)}
  load_numba_functions(os.path.join(MATH, "event", "_csr_matvec.py"),
                       ["_event_csr_matvec_transpose_numba_imp1_bool", "_event_csr_matvec_transpose_numba_imp2",
                        "_event_csr_matvec_numba_imp1_bool", "_event_csr_matvec_numba_imp2"], ns)
  load_numba_functions(os.path.join(MATH, "sparse", "_csr_mv.py"),
                       ["_csr_matvec_transpose_numba_imp", "_csr_matvec_numba_imp"], ns)
  load_numba_functions(os.path.join(MATH, "event", "_info_collection.py"), ["_event_info"], ns)
  rng = np.random.default_rng(20240601)
  out = {}
  shapes = [(100, 200), (200, 200), (200, 100), (10, 1000), (2, 10000), (1000, 10), (10000, 2), (37, 53)]
  for si, shape in enumerate(shapes):
    m, n = shape
    indices, indptr = fixed_prob_csr(rng, m, n, 0.4)
    heter = rng.normal(0.5, 0.1, size=indices.shape).astype(np.float32)
    for transpose in (1, 0):
      nev = m if transpose else n
      ev = rng.random(nev) < 0.1
      evf = np.where(rng.random(nev) < 0.5, ev.astype(np.float32), -ev.astype(np.float32) * 0.5)
      vec = rng.normal(0.0, 1.0, nev).astype(np.float32)
      key = f"{m}x{n}|T{transpose}"
      out[key + "|indices"] = indices
      out[key + "|indptr"] = indptr
      out[key + "|heter"] = heter
      out[key + "|events"] = ev
      out[key + "|events_f"] = evf
      out[key + "|vector"] = vec
      nout = n if transpose else m
      for wname, data in (("homo", np.array([-0.7], np.float32)), ("heter", heter)):
        if wname == "heter" and data.shape[0] <= 1:
          continue  # the Numba kernels treat a length-0/1 data array as homogeneous
        ins = (data, indices, indptr, ev, shape, None)
        res = np.zeros(nout, np.float32)
        fn = ns["_event_csr_matvec_transpose_numba_imp1_bool"] if transpose else ns["_event_csr_matvec_numba_imp1_bool"]
        fn(res, ins)
        out[key + f"|event_bool_{wname}"] = res
        res = np.zeros(nout, np.float32)
        fn = ns["_event_csr_matvec_transpose_numba_imp2"] if transpose else ns["_event_csr_matvec_numba_imp2"]
        fn(res, (data, indices, indptr, evf, shape, None))
        out[key + f"|event_float_{wname}"] = res
        res = np.zeros(nout, np.float32)
        fn = ns["_csr_matvec_transpose_numba_imp"] if transpose else ns["_csr_matvec_numba_imp"]
        fn(res, (data, indices, indptr, vec, shape, None))
        out[key + f"|sparse_{wname}"] = res
  for n in (1, 5, 100, 1000, 4097):
    ev = rng.random(n) < 0.3
    ids = np.zeros(n, np.int32)
    num = np.zeros(1, np.int32)
    ns["_event_info"]((ids, num), ev)
    out[f"info|{n}|events"] = ev
    out[f"info|{n}|ids"] = ids
    out[f"info|{n}|num"] = num
  return out


def gen_plasticity():
  """Weight updates of the CSR layers' STDP hook (brainpy/_src/dnn/linear.py:650-698) and the
  CSR -> CSC conversion they use (brainpy/_src/connect/base.py:645-726, numpy branch with a
  stable argsort -- the order jnp.argsort gives the jax branch)."""
  ns = {"np": np, "numba": types.SimpleNamespace(prange=range)}
  load_numba_functions(os.path.join(REF, "brainpy", "_src", "dnn", "linear.py"),
                       ["_cpu_csr_on_pre_update", "_cpu_csc_on_pre_update"], ns)
  stable_np = types.SimpleNamespace(**{k: getattr(np, k) for k in dir(np) if not k.startswith("__")})
  stable_np.argsort = lambda a: np.argsort(a, kind="stable")
  cns = {"onp": stable_np, "jnp": None, "bm": None, "get_idx_type": lambda: np.int32}
  load_functions(os.path.join(REF, "brainpy", "_src", "connect", "base.py"), ["csr2csc", "csr2coo", "coo2csc"], cns)
  rng = np.random.default_rng(20240905)
  out = {}
  for m, n, k in [(50, 80, 10), (200, 120, 30), (7, 500, 100), (300, 7, 3)]:
    indices = np.concatenate([rng.permutation(n)[:k] for _ in range(m)]).astype(np.int32)
    indptr = (np.arange(m + 1) * k).astype(np.int32)
    w = rng.normal(0.3, 0.2, indices.size).astype(np.float32)
    pre_ids, c_indptr, w_ids = cns["csr2csc"]((indices, indptr), n, data=np.arange(indices.size))
    key = f"{m}x{n}"
    out[key + "|indices"] = indices
    out[key + "|indptr"] = indptr
    out[key + "|w"] = w
    out[key + "|csc_pre_ids"] = np.asarray(pre_ids, np.int32)
    out[key + "|csc_indptr"] = np.asarray(c_indptr, np.int32)
    out[key + "|csc_w_ids"] = np.asarray(w_ids, np.int32)
    pre_spike = rng.random(m) < 0.3
    post_spike = rng.random(n) < 0.3
    post_trace = rng.normal(0.0, 0.2, n).astype(np.float32)
    pre_trace = rng.normal(0.0, 0.2, m).astype(np.float32)
    out[key + "|pre_spike"] = pre_spike
    out[key + "|post_spike"] = post_spike
    out[key + "|post_trace"] = post_trace
    out[key + "|pre_trace"] = pre_trace
    for bi, (lo, hi) in enumerate([(-np.inf, np.inf), (-0.1, 0.6), (0.0, 0.3)]):
      lo32, hi32 = np.array(lo, np.float32), np.array(hi, np.float32)
      res = np.zeros_like(w)
      ns["_cpu_csr_on_pre_update"](w, indices, indptr, pre_spike, post_trace, lo32, hi32, res)
      out[key + f"|on_pre|{bi}"] = res
      res = np.zeros_like(w)
      ns["_cpu_csc_on_pre_update"](w, out[key + "|csc_pre_ids"], out[key + "|csc_indptr"], out[key + "|csc_w_ids"],
                                   post_spike, pre_trace, lo32, hi32, res)
      out[key + f"|on_post|{bi}"] = res
  return out


# --------------------------------------------------------------------------
# consumer: LifRefLTC / LifRef, Expon, COBA, exponential Euler, VarDelay
# --------------------------------------------------------------------------
DYN = os.path.join(REF, "brainpy", "_src")


def load_class(path, cls, names, bases, ns):
  """Defines class `cls` in `ns` from the reference's own methods `names` of that class in
  `path`, on the stand-in `bases` (names looked up in ns)."""
  tree = ast.parse(open(path).read())
  node = next((n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls), None)
  if node is None:
    raise RuntimeError(f"{path}: no class {cls}")
  body = [n for n in node.body if isinstance(n, ast.FunctionDef) and n.name in names]
  if {n.name for n in body} != set(names):
    raise RuntimeError(f"{path}: {cls} lacks some of {names}")
  for n in body:
    strip_annotations(n)
  cdef = ast.ClassDef(name=cls, bases=[ast.Name(id=b, ctx=ast.Load()) for b in bases], keywords=[], body=body,
                      decorator_list=[], type_params=[])
  mod = ast.fix_missing_locations(ast.Module(body=[cdef], type_ignores=[]))
  exec(compile(mod, path, "exec"), ns)
  return ns[cls]


def load_method(path, cls, name):
  """The reference's method `name` of class `cls` as a module-level function definition."""
  tree = ast.parse(open(path).read())
  node = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls)
  fn = next(n for n in node.body if isinstance(n, ast.FunctionDef) and n.name == name)
  return strip_annotations(fn)


def strip_annotations(fn):
  """Drops decorators and type annotations (their names live in modules not loaded here)."""
  fn.decorator_list = []
  fn.returns = None
  a = fn.args
  for arg in a.posonlyargs + a.args + a.kwonlyargs + ([a.vararg] if a.vararg else []) + ([a.kwarg] if a.kwarg else []):
    arg.annotation = None
  return fn


class Dual:
  """Forward-mode dual number over float32 arrays: the stand-in for JAX's JVP inside
  bm.vector_grad (the expressions it differentiates use -, +, *, / only)."""
  __array_ufunc__ = None  # numpy operands defer to the reflected operators below

  def __init__(self, v, d):
    self.v = np.asarray(v, np.float32)
    self.d = np.asarray(d, np.float32)

  @staticmethod
  def _vd(o):
    return (o.v, o.d) if isinstance(o, Dual) else (o, None)

  def __neg__(self):
    return Dual(-self.v, -self.d)

  def __add__(self, o):
    ov, od = self._vd(o)
    return Dual(self.v + ov, self.d if od is None else self.d + od)

  __radd__ = __add__

  def __sub__(self, o):
    ov, od = self._vd(o)
    return Dual(self.v - ov, self.d if od is None else self.d - od)

  def __rsub__(self, o):
    return Dual(o - self.v, -self.d)

  def __mul__(self, o):
    ov, od = self._vd(o)
    return Dual(self.v * ov, self.d * ov if od is None else self.d * ov + self.v * od)

  def __rmul__(self, o):
    return Dual(o * self.v, o * self.d)

  def __truediv__(self, o):
    assert not isinstance(o, Dual)
    return Dual(self.v / o, self.d / o)


class NS(types.SimpleNamespace):
  pass


def consumer_namespace(state):
  """Globals of the extracted reference code, with numpy stand-ins."""
  others = {"jnp": np, "as_jax": np.asarray}
  load_functions(os.path.join(MATH, "others.py"), ["_exprel"], others)

  def exprel(x, threshold=None):  # brainpy.math.exprel: the float32 threshold 1e-5
    x = np.asarray(x, np.float32)
    return others["_exprel"](x, 1e-5 if threshold is None else threshold)

  def vector_grad(func, argnums=0, return_value=False):
    assert argnums == 0
    def g(*args, **kw):
      x = np.asarray(args[0], np.float32)
      r = func(Dual(x, np.ones_like(x)), *args[1:], **kw)
      grad, val = (r.d, r.v) if isinstance(r, Dual) else (np.zeros_like(x), np.asarray(r, np.float32))
      return (grad, val) if return_value else grad
    return g

  class TrainingMode:
    pass

  class BatchingMode:
    pass

  bm = NS(where=np.where, logical_or=np.logical_or, exprel=exprel, vector_grad=vector_grad,
          TrainingMode=TrainingMode, BatchingMode=BatchingMode,
          as_jax=lambda x, dtype=None: np.asarray(x, dtype=dtype))

  class Share:
    def load(self, key):
      return state[key]

    def __getitem__(self, key):
      return state[key]

  def get_args(f):  # integrators/utils.py:30-100: variables before `t`, the rest after it
    names = list(inspect.signature(f).parameters)
    k = names.index("t")
    return names[:k], names[k:], names

  ns = {"np": np, "bm": bm, "share": Share(), "jnp": np, "jax": NS(lax=NS(stop_gradient=lambda x: x)),
        "utils": NS(get_args=get_args), "joint_eq": NS(JointEq=type("JointEq", (), {})),
        "errors": NS(DiffEqError=ValueError), "C": NS(DT="dt", multi_vars_msg="{cls}{vars}{eq}"),
        "check": NS(is_checking=lambda: False), "jit_error": lambda *a, **k: None,
        "ROTATE_UPDATE": "rotation", "CONCAT_UPDATE": "concat", "isinstance": isinstance}
  return ns


def make_consumer_classes(ns):
  # exponential Euler (integrators/ode/exponential.py:338-364): the reference's integral
  fn = load_method(os.path.join(DYN, "integrators", "ode", "exponential.py"), "ExponentialEuler", "_build_integrator")
  exec(compile(ast.fix_missing_locations(ast.Module(body=[fn], type_ignores=[])), "exponential.py", "exec"), ns)
  build_integrator = ns["_build_integrator"]

  def odeint(f, dt):
    (integral, vars_, pars_), = build_integrator(NS(dt=dt), f)
    names = vars_ + pars_ + ["dt"]
    def integral_func(*args):  # ExponentialEuler.build's mapping of positional arguments
      kw = {names[i]: a for i, a in enumerate(args)}
      return integral(kw[names[0]], **{a: kw[a] for a in names[1:] if a in kw})
    return integral_func

  class Var:
    """bm.Variable stand-in: .value, in-place +=, and arithmetic on its value."""
    def __init__(self, value):
      self.value = value

    def __iadd__(self, x):  # Variable += x
      self.value = self.value + x
      return self

    def __array__(self, dtype=None, copy=None):
      return np.asarray(self.value, dtype=dtype)

  for op in ("add", "sub", "mul", "truediv", "le", "lt", "ge", "gt"):
    for name in (f"__{op}__", f"__r{op}__"):
      if hasattr(np.ndarray, name):
        setattr(Var, name, (lambda nm: lambda self, o: getattr(np.asarray(self.value), nm)(o))(name))
  Var.__neg__ = lambda self: -np.asarray(self.value)

  class NeuBase:  # the mixin's current and delta input sums (mixin.py:427-469)
    pass

  load_class(os.path.join(DYN, "mixin.py"), "SupportInputProj", ["sum_current_inputs", "sum_delta_inputs"], [], ns)
  ns["NeuBase"] = ns["SupportInputProj"]
  lif = os.path.join(DYN, "dyn", "neurons", "lif.py")
  load_class(lif, "LifLTC", ["derivative"], ["NeuBase"], ns)
  load_class(lif, "LifRefLTC", ["update"], ["LifLTC"], ns)
  load_class(lif, "LifRef", ["derivative", "update"], ["LifRefLTC"], ns)
  load_class(os.path.join(DYN, "dyn", "synapses", "abstract_models.py"), "Expon", ["derivative", "update", "add_current"],
             [], ns)
  load_class(os.path.join(DYN, "dyn", "outs", "outputs.py"), "COBA", ["update"], [], ns)
  load_class(os.path.join(DYN, "delay.py"), "VarDelay", ["retrieve", "update", "at"], [], ns)
  return odeint, Var


def consumer_net(ns, odeint, Var, n_exc, n_inh, ind_e, ptr_e, ind_i, ptr_i, we, wi, V0, ltc, d_e, d_i, steps,
                 trace_steps, dt=0.1, inp=20.0):
  """EICOBA_PostAlign (examples/dynamics_simulation/COBA.py:58-109) stepped with the
  reference's own update methods; the projections' products are exact counts times the weight
  (the operators are pinned by their own fixtures)."""
  n = n_exc + n_inh
  state = ns["share"].load.__self__ if False else None
  groups = {}
  for name, lo, hi in (("E", 0, n_exc), ("I", n_exc, n)):
    cls = ns["LifRefLTC"] if ltc else ns["LifRef"]
    neu = cls.__new__(cls)
    neu.V_rest, neu.V_th, neu.V_reset, neu.tau, neu.tau_ref, neu.R = -60.0, -50.0, -60.0, 20.0, 5.0, 1.0
    neu.V = Var(V0[lo:hi].astype(np.float32))
    neu.spike = Var(np.zeros(hi - lo, bool))
    neu.t_last_spike = Var(np.full(hi - lo, -1e7, np.float32))
    neu.ref_var = False
    neu.mode = None
    neu.delta_inputs = {}
    neu.integral = odeint(neu.derivative, dt)
    syn = {}
    for kind, tau, E in (("e", 5.0, 0.0), ("i", 10.0, -80.0)):
      s = ns["Expon"].__new__(ns["Expon"])
      s.tau = tau
      s.g = Var(np.zeros(hi - lo, np.float32))
      s.integral = odeint(s.derivative, dt)
      o = ns["COBA"].__new__(ns["COBA"])
      o.E = E
      syn[kind] = (s, o)
    # current inputs in registration order (E2E / E2I before I2E / I2I): excitatory first
    neu.current_inputs = {k: (lambda V, s=s, o=o: o.update(s.g.value, V)) for k, (s, o) in syn.items()}
    groups[name] = (neu, syn, lo, hi)
  delays = {}
  for name, d, lo, hi in (("E", d_e, 0, n_exc), ("I", d_i, n_exc, n)):
    if d > 0:
      dl = ns["VarDelay"].__new__(ns["VarDelay"])
      dl.method, dl.max_length, dl.mode = "rotation", d, None
      dl.data = np.zeros((d, hi - lo), bool)
      dl.target = groups[name][0].spike
      dl._registered_entries = {"proj": d}
      delays[name] = dl

  def spikes_of(name):
    if name in delays:
      return np.asarray(delays[name].at("proj"), bool)
    return groups[name][0].spike.value

  V_trace = np.zeros((trace_steps, n), np.float32)
  counts = np.zeros(steps, np.int64)
  for i in range(steps):
    SHARE.update(i=i, t=np.float32(i) * np.float32(dt), dt=dt)
    # projections (update order E2I, I2I, I2E, E2E): g += count * w, per post group
    dge = np.zeros(n, np.float32)
    dgi = np.zeros(n, np.float32)
    for pre, ind, ptr, w, acc in (("E", ind_e, ptr_e, we, dge), ("I", ind_i, ptr_i, wi, dgi)):
      act = np.nonzero(spikes_of(pre))[0]
      cnt = np.zeros(n, np.int64)
      for r in act:
        np.add.at(cnt, ind[ptr[r]:ptr[r + 1]], 1)
      acc += cnt.astype(np.float32) * np.float32(w)
    for name, (neu, syn, lo, hi) in groups.items():
      syn["e"][0].add_current(dge[lo:hi])
      syn["i"][0].add_current(dgi[lo:hi])
    # each group: its synapses decay (before-updates), then the neurons integrate
    for name, (neu, syn, lo, hi) in groups.items():
      syn["e"][0].update()
      syn["i"][0].update()
      neu.update(np.float32(inp))
    for name, dl in delays.items():
      dl.update()
    V = np.concatenate([groups["E"][0].V.value, groups["I"][0].V.value])
    sp = np.concatenate([groups["E"][0].spike.value, groups["I"][0].spike.value])
    counts[i] = int(sp.sum())
    if i < trace_steps:
      V_trace[i] = V
  return V_trace, counts


SHARE = {}


def gen_consumer():
  global SHARE
  ns = consumer_namespace(SHARE)
  odeint, Var = make_consumer_classes(ns)
  rng = np.random.default_rng(2024)
  n_exc, n_inh = 160, 40
  n = n_exc + n_inh
  out = {}

  def fixed_rows(m, K):
    ptr = np.arange(0, m * K + 1, K, dtype=np.int32)
    ind = np.concatenate([rng.choice(n, K, replace=False) for _ in range(m)]).astype(np.int32)
    return ind, ptr

  ind_e, ptr_e = fixed_rows(n_exc, 10)
  ind_i, ptr_i = fixed_rows(n_inh, 10)
  V0 = rng.normal(-55.0, 5.0, n).astype(np.float32)
  out.update(ind_e=ind_e, ptr_e=ptr_e, ind_i=ind_i, ptr_i=ptr_i, V0=V0,
             sizes=np.array([n_exc, n_inh], np.int64), weights=np.array([0.6, 6.7], np.float32))
  for tag, ltc, de, di in (("ltc", True, 0, 0), ("lifref", False, 0, 0), ("ltc_d3_1", True, 3, 1), ("ltc_d2_0", True, 2, 0)):
    Vt, counts = consumer_net(ns, odeint, Var, n_exc, n_inh, ind_e, ptr_e, ind_i, ptr_i, 0.6, 6.7, V0, ltc, de, di,
                              steps=300, trace_steps=100)
    out[f"{tag}|V"] = Vt
    out[f"{tag}|counts"] = counts
    out[f"{tag}|cfg"] = np.array([int(ltc), de, di], np.int64)
  # VarDelay's rotating indices alone: what step's value each delay reads at each step
  for L in (1, 3, 5):
    for d in range(1, L + 1):
      dl = ns["VarDelay"].__new__(ns["VarDelay"])
      dl.method, dl.max_length, dl.mode = "rotation", L, None
      dl.data = np.full((L, 1), -1, np.int64)
      dl.target = Var(np.zeros(1, np.int64))
      dl._registered_entries = {"x": d}
      read = []
      for i in range(24):
        SHARE.update(i=i)
        read.append(int(np.asarray(dl.at("x"))[0]))
        dl.target.value = np.array([i], np.int64)  # the value step i produces
        dl.update()
      out[f"delay|L{L}|d{d}"] = np.array(read, np.int64)
  return out


def main():
  np.seterr(over="ignore")
  pl = gen_plasticity()
  np.savez_compressed(os.path.join(HERE, "plasticity.npz"), **pl)
  print("plasticity:", len(pl), "arrays")
  lf = gen_lfsr()
  np.savez_compressed(os.path.join(HERE, "lfsr88.npz"), **lf)
  print("lfsr88:", len(lf), "arrays")
  cs = gen_csr()
  np.savez_compressed(os.path.join(HERE, "csr.npz"), **cs)
  print("csr:", len(cs), "arrays")
  jc = gen_jitconn()
  np.savez_compressed(os.path.join(HERE, "jitconn.npz"), **jc)
  n_conn = sum(v.size for k, v in jc.items() if k.endswith("|rows"))
  print("jitconn:", len(jc), "arrays,", n_conn, "connections")
  co = gen_consumer()
  np.savez_compressed(os.path.join(HERE, "consumer.npz"), **co)
  print("consumer:", len(co), "arrays")


if __name__ == "__main__":
  main()
