"""The jitconn transpose rule on the oracle (no GPU).

The reference differentiates y = M v with respect to v by regenerating the matrix with
transpose and outdim_parallel both flipped (brainpy/_src/math/jitconn/_matvec_taichi.py:148-158),
relying on "the M in f(outdim_parallel=True, transpose=False) is the M^T in
f(outdim_parallel=False, transpose=True)" (_matvec_taichi.py:270-279).  These tests pin where
that holds: exactly for the Taichi CPU connectivity (one stream per owner over the whole other
dimension), and not for the Taichi GPU connectivity, whose 32 lanes per owner split a width
computed from the owner count."""
import pytest


def _conn(orc, kind, p0, p1, prob, seed, nr, nc, odp, variant):
  from brainpy_gb300.math.jitconn import conn_len
  r, c, w = orc.jitconn_connections(kind, p0, p1, conn_len(prob), seed, nr, nc, odp, variant)
  return r, c, w


@pytest.mark.parametrize("kind,p0,p1", [("homo", 0.8, 0.0), ("uniform", -0.5, 1.5), ("normal", 0.2, 0.9)])
@pytest.mark.parametrize("shape,prob", [((300, 200), 0.05), ((64, 1000), 0.1), ((2048, 4096), 0.01)])
@pytest.mark.parametrize("odp", [True, False])
def test_flipped_call_is_transpose_for_cpu_connectivity(orc, kind, p0, p1, shape, prob, odp):
  a, b = shape
  r, c, w = _conn(orc, kind, p0, p1, prob, 1234, a, b, odp, "cpu")
  r2, c2, w2 = _conn(orc, kind, p0, p1, prob, 1234, b, a, not odp, "cpu")
  assert sorted(zip(r.tolist(), c.tolist(), w.tolist())) == sorted(zip(c2.tolist(), r2.tolist(), w2.tolist()))


def test_flipped_call_differs_for_gpu_connectivity(orc):
  r, c, _ = _conn(orc, "homo", 1.0, 0.0, 0.1, 1234, 64, 1000, True, "gpu")
  r2, c2, _ = _conn(orc, "homo", 1.0, 0.0, 0.1, 1234, 1000, 64, False, "gpu")
  # 64 owners: lanes of width (64 + 1) >> 5 = 2 cover 64 of the 1000 columns
  assert c.max() < 64 and r.size < 200
  assert sorted(zip(r.tolist(), c.tolist())) != sorted(zip(c2.tolist(), r2.tolist()))
