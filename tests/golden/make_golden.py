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


if __name__ == "__main__":
  main()
