"""A minimal stand-in for the ``taichi`` module, used only to execute the
reference's own Taichi kernel source in plain Python when generating golden
fixtures (Taichi is not installable here).

What is emulated:

* ``@ti.kernel`` / ``@ti.func`` run as ordinary Python functions, loops serial;
* integer scalars carry a width and signedness; a mixed binary operation takes
  the type C++ gives ``decltype(a + b)`` (Taichi derives its promotion table
  from exactly that), so ``u32 op i32 -> u32`` with 32-bit wrap-around;
* Python int literals are ``i32`` and Python float literals ``f32``
  (Taichi's default_ip / default_fp);
* float arithmetic is numpy float32; ``ti.log/sin/sqrt`` use numpy float32.

``ndarray`` arguments are supplied by the generator (plain numpy arrays or the
tracing wrappers in make_golden.py).
"""
import math
import types

import numpy as np


class TInt:
  __slots__ = ("v", "bits", "signed")

  def __init__(self, v, bits=32, signed=True):
    mask = (1 << bits) - 1
    v = int(v) & mask
    if signed and v >= (1 << (bits - 1)):
      v -= 1 << bits
    self.v, self.bits, self.signed = v, bits, signed

  # -- promotion ------------------------------------------------------------
  @staticmethod
  def _as(o):
    if isinstance(o, TInt):
      return o
    if isinstance(o, (bool, np.bool_)):
      return TInt(int(o), 32, True)
    if isinstance(o, (int, np.integer)):
      if isinstance(o, np.integer):
        return TInt(int(o), o.dtype.itemsize * 8, np.issubdtype(o.dtype, np.signedinteger))
      return TInt(o, 32, True)
    return None

  @staticmethod
  def _promote(a, b):
    bits = max(a.bits, b.bits)
    if a.bits == b.bits:
      signed = a.signed and b.signed
    else:
      wide = a if a.bits > b.bits else b
      signed = wide.signed
    return bits, signed

  def _bin(self, o, fn, rev=False):
    oi = TInt._as(o)
    if oi is None:  # float operand
      f = np.float32(self.v)
      of = np.float32(o) if not isinstance(o, np.floating) else o
      return fn(of, f) if rev else fn(f, of)
    bits, signed = TInt._promote(self, oi)
    a, b = TInt(self.v, bits, signed), TInt(oi.v, bits, signed)
    if rev:
      a, b = b, a
    return TInt(fn(a.v, b.v), bits, signed)

  def __add__(self, o): return self._bin(o, lambda a, b: a + b)
  def __radd__(self, o): return self._bin(o, lambda a, b: a + b, True)
  def __sub__(self, o): return self._bin(o, lambda a, b: a - b)
  def __rsub__(self, o): return self._bin(o, lambda a, b: a - b, True)
  def __mul__(self, o): return self._bin(o, lambda a, b: a * b)
  def __rmul__(self, o): return self._bin(o, lambda a, b: a * b, True)

  def __mod__(self, o):
    def f(a, b):  # C++ truncated remainder
      r = abs(a) % abs(b)
      return -r if a < 0 else r
    return self._bin(o, f)

  def __and__(self, o): return self._bin(o, lambda a, b: a & b)
  def __rand__(self, o): return self._bin(o, lambda a, b: a & b, True)
  def __or__(self, o): return self._bin(o, lambda a, b: a | b)
  def __xor__(self, o): return self._bin(o, lambda a, b: a ^ b)
  def __rxor__(self, o): return self._bin(o, lambda a, b: a ^ b, True)

  def __lshift__(self, o):
    return TInt(self.v << int(o), self.bits, self.signed)

  def __rshift__(self, o):
    s = int(o)
    if self.signed:
      return TInt(self.v >> s, self.bits, True)
    return TInt((self.v & ((1 << self.bits) - 1)) >> s, self.bits, False)

  def _cmp(self, o, fn):
    oi = TInt._as(o)
    if oi is None:
      return fn(float(self.v), float(o))
    bits, signed = TInt._promote(self, oi)
    return fn(TInt(self.v, bits, signed).v, TInt(oi.v, bits, signed).v)

  def __lt__(self, o): return self._cmp(o, lambda a, b: a < b)
  def __le__(self, o): return self._cmp(o, lambda a, b: a <= b)
  def __gt__(self, o): return self._cmp(o, lambda a, b: a > b)
  def __ge__(self, o): return self._cmp(o, lambda a, b: a >= b)
  def __eq__(self, o): return self._cmp(o, lambda a, b: a == b)
  def __ne__(self, o): return self._cmp(o, lambda a, b: a != b)
  def __hash__(self): return hash(self.v)
  def __index__(self): return self.v
  def __int__(self): return self.v
  def __bool__(self): return self.v != 0
  def __repr__(self): return f"{'i' if self.signed else 'u'}{self.bits}({self.v})"


def _dtype_caster(bits, signed):
  def cast(x):
    if isinstance(x, TInt):
      return TInt(x.v, bits, signed)
    if isinstance(x, (float, np.floating)):
      return TInt(int(math.trunc(float(x))), bits, signed)
    return TInt(int(x), bits, signed)
  cast.bits, cast.signed = bits, signed
  return cast


u32 = uint32 = _dtype_caster(32, False)
i32 = int32 = _dtype_caster(32, True)
u64 = _dtype_caster(64, False)
i64 = _dtype_caster(64, True)


def f32(x):
  if isinstance(x, TInt):
    return np.float32(x.v)
  return np.float32(x)


float32 = f32


def cast(x, dtype):
  return dtype(x)


def _max(a, b):
  return a if a >= b else b  # only used on like-typed operands in the kernels


def _min(a, b):
  if isinstance(a, TInt) or isinstance(b, TInt):
    ai, bi = TInt._as(a), TInt._as(b)
    bits, signed = TInt._promote(ai, bi)
    ai, bi = TInt(ai.v, bits, signed), TInt(bi.v, bits, signed)
    return ai if ai.v <= bi.v else bi
  return a if a <= b else b


def _max_typed(a, b):
  if isinstance(a, TInt) or isinstance(b, TInt):
    ai, bi = TInt._as(a), TInt._as(b)
    bits, signed = TInt._promote(ai, bi)
    ai, bi = TInt(ai.v, bits, signed), TInt(bi.v, bits, signed)
    return ai if ai.v >= bi.v else bi
  if isinstance(a, (float, np.floating)) or isinstance(b, (float, np.floating)):
    a, b = np.float32(a), np.float32(b)
  if isinstance(a, int) and isinstance(b, int):
    return TInt(max(a, b), 32, True)
  return a if a >= b else b


def _uvec4(a, b, c, d):
  return [u32(a), u32(b), u32(c), u32(d)]


def _log(x): return np.log(np.float32(x), dtype=np.float32)
def _sin(x): return np.sin(np.float32(x), dtype=np.float32)
def _sqrt(x): return np.sqrt(np.float32(x), dtype=np.float32)


def _identity_decorator(fn=None, **kwargs):
  if fn is None:
    return lambda f: f
  return fn


class _Types:
  @staticmethod
  def ndarray(*a, **k): return object
  @staticmethod
  def vector(*a, **k): return object


def make_module():
  ti = types.ModuleType("taichi")
  ti.kernel = _identity_decorator
  ti.func = _identity_decorator
  ti.u32 = ti.uint32 = u32
  ti.i32 = ti.int32 = i32
  ti.u64 = u64
  ti.i64 = i64
  ti.f32 = ti.float32 = f32
  ti.cast = cast
  ti.max = _max_typed
  ti.min = _min
  ti.log = _log
  ti.sin = _sin
  ti.sqrt = _sqrt
  ti.loop_config = lambda **k: None
  ti.types = _Types()
  math_ns = types.SimpleNamespace(uvec4=_uvec4, pi=math.pi)
  ti.math = math_ns
  return ti
