"""On-device construction of FixedProb connectivity.

``FixedProb`` mirrors ``bp.conn.FixedProb`` (brainpy/_src/connect/random_conn.py:30-128) and
``fixed_prob_csr`` is its fixed-fan-out core: every pre-synaptic row gets K distinct,
uniformly random post-synaptic columns (the law of numba's ``rng.choice(num_post, K,
replace=False)``), generated in HBM by ``bp_fixed_prob_fill`` from a counter-based sequence
seeded by (seed, row).  The reference's numba stream itself cannot be reproduced; its law is.

``bernoulli_events`` and ``normal_weights`` are counter-based synthetic inputs for tests and
benchmarks.
"""
import math

import numpy as np
import torch

_M64 = (1 << 63) - 1


def _mix(x):
  """SplitMix64-style finaliser on int64 tensors (wrap-around arithmetic)."""
  x = x ^ (x >> 30)
  x = x * -4658895280553007687  # 0xbf58476d1ce4e5b9 as signed int64
  x = x ^ (x >> 27)
  x = x * -7723592293110705685  # 0x94d049bb133111eb as signed int64
  x = x ^ (x >> 31)
  return x & _M64


def _gpu_device(device):
  """The CUDA device the generator runs on: `device` itself, or the current CUDA device when
  the arrays are wanted elsewhere (they are built on the GPU and copied)."""
  if device is not None and torch.device(device).type == "cuda":
    return torch.device(device)
  if not torch.cuda.is_available():
    raise RuntimeError("the FixedProb generator runs on a CUDA device (sm_103a); none is available")
  return torch.device("cuda", torch.cuda.current_device())


def _fixed_prob_device(m, n, K, seed, allow_multi, include_self, mask, dev):
  """(indices int32, indptr int64) of the device generator, on CUDA device `dev`."""
  from . import _lib
  if dev.type != "cuda":
    raise ValueError(f"the generator's arrays must live on a CUDA device, not {dev}")
  L = _lib.lib()
  st = _lib.stream_handle(dev)
  if mask is None and include_self:
    indptr = torch.arange(m + 1, dtype=torch.int64, device=dev) * K
  else:
    lengths = torch.empty(m, dtype=torch.int32, device=dev)
    _lib.check(L.bp_fixed_prob_row_lengths(m, n, K, seed, int(allow_multi), int(include_self),
                                           _lib.ptr(mask) if mask is not None else None, _lib.ptr(lengths), st),
               "fixed_prob_row_lengths")
    if m and int(lengths.min()) < 0:
      raise RuntimeError("FixedProb: a row overran its draw bound")
    indptr = torch.zeros(m + 1, dtype=torch.int64, device=dev)
    indptr[1:] = torch.cumsum(lengths.to(torch.int64), 0)
  nnz = int(indptr[-1]) if m else 0
  indices = torch.empty(nnz, dtype=torch.int32, device=dev)
  _lib.check(L.bp_fixed_prob_fill(m, n, K, seed, int(allow_multi), int(include_self),
                                  _lib.ptr(mask) if mask is not None else None, _lib.ptr(indptr), _lib.ptr(indices), st),
             "fixed_prob_fill")
  if nnz and int(indices.min()) < 0:
    raise RuntimeError("FixedProb: a row overran its draw bound")
  return indices, indptr


def fixed_prob_csr(num_pre, num_post, fan_out, seed=0, device=None, index_dtype=torch.int32):
  """(indices, indptr) on `device` of a num_pre x num_post CSR whose rows hold `fan_out`
  distinct uniformly random columns (FixedProb with K = fan_out, include_self=True)."""
  K = int(fan_out)
  if K < 0 or K > num_post:
    raise ValueError(f"fan_out {K} must lie in [0, num_post={num_post}]")
  gpu = _gpu_device(device)
  indices, indptr = _fixed_prob_device(int(num_pre), int(num_post), K, int(seed), False, True, None, gpu)
  target = gpu if device is None else torch.device(device)
  return indices.to(index_dtype).to(target), indptr.to(index_dtype).to(target)


class FixedProb:
  """``bp.conn.FixedProb(prob, pre_ratio, include_self, allow_multi_conn, seed)`` built on the
  GPU (brainpy/_src/connect/random_conn.py:30-128).

  Every selected pre-synaptic row gets ``K = int(post_num * prob)`` post-synaptic columns:
  distinct and uniformly random (the law of numba's ``rng.choice(post_num, K,
  replace=False)``), or K independent uniform draws with ``allow_multi_conn``.  With
  ``include_self=False`` the drawn diagonal entries are removed afterwards, as in the
  reference.  ``bp_fixed_prob_fill`` generates the rows from a counter-based sequence, so the
  same seed gives the same connectivity on every device; the reference's numba stream itself
  cannot be reproduced.

  ``pre_ratio < 1`` selects ``int(pre_num * pre_ratio)`` rows uniformly without replacement;
  the other rows are empty.  (The reference's build_csr returns a CSR with only the selected
  rows, in random order, which loses which pre-synaptic neuron each row belongs to.)
  """

  def __init__(self, prob, pre_ratio=1., include_self=True, allow_multi_conn=False, seed=None, device=None):
    if not 0. <= prob <= 1.:
      raise ValueError(f"prob must lie in [0, 1], got {prob}")
    if not 0. <= pre_ratio <= 1.:
      raise ValueError(f"pre_ratio must lie in [0, 1], got {pre_ratio}")
    self.prob = float(prob)
    self.pre_ratio = float(pre_ratio)
    self.include_self = bool(include_self)
    self.allow_multi_conn = bool(allow_multi_conn)
    self.seed = int(np.random.randint(0, 2 ** 31 - 1)) if seed is None else int(seed)
    self.device = device
    self.pre_num = self.post_num = None
    self._csr = None

  def __repr__(self):
    return (f"{self.__class__.__name__}(prob={self.prob}, pre_ratio={self.pre_ratio}, "
            f"include_self={self.include_self}, allow_multi_conn={self.allow_multi_conn}, seed={self.seed})")

  def __call__(self, pre_size, post_size=None):
    post_size = pre_size if post_size is None else post_size
    self.pre_num = int(np.prod(pre_size))
    self.post_num = int(np.prod(post_size))
    self._csr = None
    return self

  def _device(self):
    return _gpu_device(self.device)

  def build_csr(self):
    """(indices, indptr), int32, on the device."""
    if self.pre_num is None:
      raise ValueError("call the connector with (pre_size, post_size) first")
    m, n = self.pre_num, self.post_num
    if not self.include_self and m != n:
      raise ValueError(f"We found pre_num != post_num ({m} != {n}). But `include_self` is set to True.")
    K = int(n * self.prob)
    dev = self._device()
    mask = None
    if self.pre_ratio < 1.:
      n_sel = int(m * self.pre_ratio)
      keys = _hash_u01(m, self.seed ^ 0x5DEECE66D, dev)
      mask = torch.zeros(m, dtype=torch.uint8, device=dev)
      if n_sel > 0:
        mask[torch.topk(keys, n_sel, largest=False).indices] = 1
    indices, indptr = _fixed_prob_device(m, n, K, self.seed, self.allow_multi_conn, self.include_self, mask, dev)
    target = dev if self.device is None else torch.device(self.device)
    return indices.to(target), indptr.to(torch.int32).to(target)

  def build_coo(self):
    """(pre_ids, post_ids), int32."""
    from .math.sparse import csr_to_coo
    indices, indptr = self.require("csr")
    return csr_to_coo(indices, indptr)

  def require(self, *structs):
    """'csr' / 'pre2post' -> (indices, indptr); 'coo' / 'ij' -> (pre_ids, post_ids)."""
    out = []
    for s in structs:
      if s in ("csr", "pre2post"):
        if self._csr is None:
          self._csr = self.build_csr()
        out.append(self._csr)
      elif s in ("coo", "ij"):
        out.append(self.build_coo())
      else:
        raise ValueError(f"unsupported structure {s!r} (csr, pre2post, coo, ij)")
    return out[0] if len(out) == 1 else tuple(out)


def csr2csc(indices, indptr, post_num):
  """(pre_ids, indptr, w_ids) of the CSC form of a CSR connection, as
  brainpy/_src/connect/base.py:645-726 with data = arange(nnz): entries sorted by column,
  row order kept within a column; pre_ids are the rows, w_ids the CSR positions.  A one-time
  setup conversion (the COO rows from bp_csr_to_coo, then torch's stable sort)."""
  from .math.sparse import csr_to_coo
  rows, cols = csr_to_coo(indices, indptr)
  order = torch.sort(cols.to(torch.int64), stable=True).indices
  dt = indices.dtype
  pre_ids = rows[order].to(dt)
  counts = torch.bincount(cols.to(torch.int64), minlength=int(post_num))[:int(post_num)]
  c_indptr = torch.zeros(int(post_num) + 1, dtype=torch.int64, device=indices.device)
  c_indptr[1:] = torch.cumsum(counts, 0)
  return pre_ids, c_indptr.to(dt), order.to(dt)


def _hash_u01(n, seed, device):
  """Counter-based uniforms in [0, 1) (float64), identical on every device."""
  i = torch.arange(n, device=device, dtype=torch.int64)
  h = _mix(i * 0x3C6EF372 + ((int(seed) * 0x9E3779B1 + 0x7F4A7C15) & _M64))
  return (h >> 11).to(torch.float64) * (1.0 / (1 << 52))


def bernoulli_events(n, rate, seed, device=None):
  """bool spike vector with P(event) = rate (counter-based, device independent)."""
  if device is None:
    device = torch.device("cuda")
  return _hash_u01(n, seed, device) < rate


def normal_weights(n, mean, std, seed, device=None, chunk=1 << 26):
  """float32 N(mean, std) weights by Box-Muller on counter-based uniforms."""
  if device is None:
    device = torch.device("cuda")
  out = torch.empty(n, dtype=torch.float32, device=device)
  for a in range(0, n, chunk):
    b = min(n, a + chunk)
    i = torch.arange(a, b, device=device, dtype=torch.int64)
    s = (int(seed) * 0x9E3779B1 + 0x2F0B7A15) & _M64
    u1 = ((_mix(i * 0x3C6EF372 + s) >> 11).to(torch.float64) + 1.0) * (1.0 / (1 << 52))
    u2 = (_mix(i * 0x6A09E667 + s) >> 11).to(torch.float64) * (1.0 / (1 << 52))
    z = torch.sqrt(-2.0 * torch.log(u1)) * torch.cos(2.0 * math.pi * u2)
    out[a:b] = (z * std + mean).to(torch.float32)
  return out
