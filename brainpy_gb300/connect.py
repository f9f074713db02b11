"""On-device construction of fixed-fan-out random CSR connectivity.

`fixed_prob_csr` builds the shape of ``bp.conn.FixedProb(prob).require('pre2post')``
(brainpy/_src/connect/random_conn.py:118-128: every pre-synaptic row gets exactly
``int(num_post * prob)`` distinct post-synaptic columns, in no particular order)
directly in HBM, from a seed.  The reference draws each row with numba's RNG, which
cannot be reproduced; this generator is our own:

* the post range is cut into K = fan-out equal strata of width ``num_post // K``;
* row r takes one column per stratum, uniform within the stratum, from a
  counter-based hash of (seed, r, k);
* the strata are visited in a per-row permuted order k -> (a_r k + b_r) mod K with
  a_r coprime to K, so a row's columns are distinct and unsorted.
"""
import math

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


def fixed_prob_csr(num_pre, num_post, fan_out, seed=0, device=None, index_dtype=torch.int32, chunk_rows=1 << 15):
  """Returns (indices, indptr) on `device` for a num_pre x num_post CSR with exactly
  `fan_out` distinct columns per row."""
  if device is None:
    device = torch.device("cuda")
  K = int(fan_out)
  if K < 0 or K > num_post:
    raise ValueError(f"fan_out {K} must lie in [0, num_post={num_post}]")
  indptr = (torch.arange(num_pre + 1, device=device, dtype=torch.int64) * K).to(index_dtype)
  if K == 0 or num_pre == 0:
    return torch.zeros(0, dtype=index_dtype, device=device), indptr
  bw = num_post // K
  cands = torch.tensor([a for a in range(1, K + 1) if math.gcd(a, K) == 1], dtype=torch.int64, device=device)
  indices = torch.empty(num_pre * K, dtype=index_dtype, device=device)
  k = torch.arange(K, device=device, dtype=torch.int64)[None, :]
  s = (int(seed) * 0x9E3779B1 + 0x632BE5AB) & _M64
  for r0 in range(0, num_pre, chunk_rows):
    r1 = min(num_pre, r0 + chunk_rows)
    r = torch.arange(r0, r1, device=device, dtype=torch.int64)[:, None]
    hr = _mix(r * 0x2545F491 + s)
    a = cands[hr % cands.numel()]
    b = _mix(hr + 0x1B873593) % K
    kp = (a * k + b) % K
    off = _mix(hr ^ (k * 0x5851F42D + 0x14057B7E)) % bw
    indices[r0 * K:r1 * K] = (kp * bw + off).reshape(-1).to(index_dtype)
  return indices, indptr


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
