"""The CPU oracle against golden vectors produced by the reference's own kernel
source (tests/golden/make_golden.py).  No GPU involved."""
import numpy as np
import pytest

from golden_util import csr_keys, jitconn_keys, load, scaled_err


def test_lfsr88_streams(orc):
  g = load("lfsr88")
  for k in g.files:
    parts = k.split("|")
    kind, seed = parts[0], int(parts[1])
    ref = g[k]
    if kind == "randint":
      np.testing.assert_array_equal(orc.lfsr88_stream(seed, 16), ref, err_msg=k)
    elif kind == "random_integers":
      got = np.array(orc.lfsr88_sequence(seed, 16, "random_integers", int(parts[2]), int(parts[3])), np.int32)
      np.testing.assert_array_equal(got, ref, err_msg=k)
    elif kind == "uniform":
      got = np.array(orc.lfsr88_sequence(seed, 16, "uniform", float(parts[2]), float(parts[3])), np.float32)
      np.testing.assert_array_equal(got, ref, err_msg=k)
    else:  # normal: libm logf/sinf vs numpy float32 -> within a few ulp
      got = np.array(orc.lfsr88_sequence(seed, 16, "normal", float(parts[2]), float(parts[3])), np.float32)
      np.testing.assert_allclose(got, ref, rtol=2e-6, atol=2e-6, err_msg=k)


def test_lfsr88_hand_checked_first_steps(orc):
  # seed 0: key = (1, 7, 15, 0); hand evaluation of tifunc.py:80-86 for one step:
  #  b = ((1<<13)^1)>>19 = 0;  s1 = ((1 & ~1) << 12) ^ 0 = 0
  #  b = ((7<<2)^7)>>25 = 0;   s2 = ((7 & ~7) << 4) ^ 0 = 0
  #  b = ((15<<3)^15)>>11 = 0; s3 = ((15 & ~15) << 17) ^ 0 = 0
  # so the first output of seed 0 is 0 (the documented small-seed degeneracy).
  assert orc.lfsr88_stream(0, 1)[0] == 0
  # seed 42: key = (43, 49, 57, 0)
  k0, k1, k2 = 43, 49, 57
  M = 0xFFFFFFFF
  b = (((k0 << 13) & M) ^ k0) >> 19
  s1 = (((k0 & 4294967294) << 12) & M) ^ b
  b = (((k1 << 2) & M) ^ k1) >> 25
  s2 = (((k1 & 4294967288) << 4) & M) ^ b
  b = (((k2 << 3) & M) ^ k2) >> 11
  s3 = (((k2 & 4294967280) << 17) & M) ^ b
  assert orc.lfsr88_stream(42, 1)[0] == (s1 ^ s2 ^ s3)


@pytest.fixture(scope="module")
def jc():
  return load("jitconn")


def test_jitconn_connectivity_bit_exact(orc, jc):
  n_conn = 0
  for key in jitconn_keys(jc):
    kind, _, _, odp, dev, _ = key.split("|")
    nr, nc, clen, seed = (int(x) for x in jc[key + "|meta"])
    p0, p1 = (float(x) for x in jc[key + "|par"])
    rows, cols, w = orc.jitconn_connections(kind, p0, p1, clen, seed, nr, nc, odp == "odp1", dev)
    np.testing.assert_array_equal(rows, jc[key + "|rows"], err_msg=key)
    np.testing.assert_array_equal(cols, jc[key + "|cols"], err_msg=key)
    W = jc[key + "|w"]
    known = ~np.isnan(W)
    if kind == "normal":
      np.testing.assert_allclose(w[known], W[known], rtol=4e-6, atol=4e-6, err_msg=key)
    else:
      np.testing.assert_array_equal(w[known], W[known], err_msg=key)
    n_conn += rows.size
  assert n_conn > 100000


def test_jitconn_gpu_stripe_quirks(orc):
  """Properties of the Taichi GPU algorithm the kernels must reproduce: lane `l` of an
  owner only reaches [step*l, step*(l+1)-2], so indices step*k-1 and >= 32*step-1 never
  connect, and an output shorter than 63 gets no connections at all."""
  rows, cols, _ = orc.jitconn_connections("homo", 1.0, 0.0, 3, 7, 100, 300, True, "gpu")
  step = max((100 + 1) >> 5, 1)
  assert cols.size > 0 and cols.max() < 32 * step - 1
  assert not np.any((cols + 1) % step == 0)
  rows, cols, _ = orc.jitconn_connections("homo", 1.0, 0.0, 3, 7, 62, 300, True, "gpu")
  assert rows.size == 0


def test_jitconn_mv_matches_connection_list(orc):
  rng = np.random.default_rng(0)
  for kind, p0, p1 in (("homo", 0.7, 0.0), ("uniform", -1.0, 2.0), ("normal", 0.3, 1.1)):
    for odp in (True, False):
      nr, nc = 333, 257
      vec = rng.normal(size=nc).astype(np.float32)
      y64, _ = orc.jitconn_mv(kind, vec, nr, p0, p1, 19, 99, odp, "gpu")
      rows, cols, w = orc.jitconn_connections(kind, p0, p1, 19, 99, nr, nc, odp, "gpu")
      ref = np.zeros(nr)
      np.add.at(ref, rows, w.astype(np.float64) * vec[cols])
      np.testing.assert_allclose(y64, ref, rtol=1e-12, atol=1e-12)


@pytest.fixture(scope="module")
def cs():
  return load("csr")


def test_event_and_sparse_csrmv(orc, cs):
  for key in csr_keys(cs):
    shp, t = key.split("|")
    m, n = (int(x) for x in shp.split("x"))
    transpose = t == "T1"
    ind, ptr = cs[key + "|indices"], cs[key + "|indptr"]
    for wname in ("homo", "heter"):
      if key + f"|event_bool_{wname}" not in cs.files:
        continue
      data = np.array([-0.7], np.float32) if wname == "homo" else cs[key + "|heter"]
      for kind, vec in (("event_bool", cs[key + "|events"]), ("event_float", cs[key + "|events_f"]),
                        ("sparse", cs[key + "|vector"])):
        ref = cs[key + f"|{kind}_{wname}"]
        if kind == "sparse":
          r = orc.csrmv(data, ind, ptr, vec, (m, n), transpose)
        else:
          r = orc.event_csrmv(data, ind, ptr, vec, (m, n), transpose, ev_rule=orc.EV_F32_POS)
        assert scaled_err(ref, r["out64"], r["abs64"]) < 1e-5, (key, kind, wname)
        if transpose:  # serial loops in the same order -> bit-exact float32
          np.testing.assert_array_equal(r["out32"], ref, err_msg=f"{key} {kind} {wname}")


def test_event_info(orc, cs):
  for n in (1, 5, 100, 1000, 4097):
    ids, num = orc.event_info(cs[f"info|{n}|events"])
    np.testing.assert_array_equal(ids, cs[f"info|{n}|ids"])
    assert num == cs[f"info|{n}|num"][0]


def test_homo_count_form_close_to_reference_order(orc, cs):
  key = "200x200|T1"
  r = orc.event_csrmv(np.array([0.6], np.float32), cs[key + "|indices"], cs[key + "|indptr"],
                      cs[key + "|events"], (200, 200), True)
  assert scaled_err(r["count32"], r["out64"], r["abs64"]) < 1e-6
  assert scaled_err(r["out32"], r["out64"], r["abs64"]) < 1e-5
