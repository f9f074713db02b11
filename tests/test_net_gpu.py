"""E/I COBA networks on the GPU against the oracle.

Event counts are exact integers and the neuron update is evaluated in the same float32
operation order on both sides, so the simulated trajectories must agree bit for bit:
membrane potentials of the first 100 steps and spike counts of every step."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dyn(bplib):
  import brainpy_gb300.dyn as d
  return d


def _oracle_split(net):
  ind = net.indices.cpu().numpy().astype(np.int32)
  ptr = net.indptr.cpu().numpy().astype(np.int64)
  ne = net.n_exc
  e_end = int(ptr[ne])
  exc_ptr = ptr[: ne + 1].astype(np.int32)
  inh_ptr = (ptr[ne:] - e_end).astype(np.int32)
  return exc_ptr, np.ascontiguousarray(ind[:e_end]), inh_ptr, np.ascontiguousarray(ind[e_end:])


def _oracle_run(orc, net, state, steps, trace_steps=0, step0=0):
  p = net.params
  op = orc.lif_params(p.V_rest, p.V_th, p.V_reset, p.tau, p.tau_ref, p.R, p.tau_e, p.tau_i, p.E_e, p.E_i, p.input,
                      p.ltc)
  ep, ei, ip, ii = _oracle_split(net)
  return orc.coba_net_run(op, net.n, net.n_exc, ep, ei, np.float32(net.we), ip, ii, np.float32(net.wi), state,
                          step0, steps, np.float32(0.1), count_mode=True, trace_steps=trace_steps)


def _v0(n, seed=3):
  return np.random.default_rng(seed).normal(-55.0, 5.0, n).astype(np.float32)


@pytest.mark.parametrize("ltc", [True, False])
def test_coba_4000_bit_exact(dyn, orc, ltc):
  """The COBA example network (3200 E + 800 I, 2 % FixedProb, we 0.6, wi 6.7)."""
  V0 = _v0(4000)
  net = dyn.EINetwork.fixed_prob(3200, 800, prob=0.02, seed=1, params=dyn.LifParams(ltc=ltc), V0=V0)
  state = net.state_numpy()
  counts, trace = net.run(1000, method="cluster", v_trace_steps=100)
  rc, rtrace = _oracle_run(orc, net, state, 1000, trace_steps=100)
  np.testing.assert_array_equal(trace.cpu().numpy(), rtrace)  # V within 0 mV over the first 100 steps
  np.testing.assert_array_equal(counts.cpu().numpy(), rc)
  got = net.state_numpy()
  for k in ("V", "ge", "gi", "t_last", "spike"):
    np.testing.assert_array_equal(got[k], state[k], err_msg=k)
  assert rc.sum() > 1000  # the network is active


def test_ops_path_and_graph_match_cluster(dyn):
  V0 = _v0(4000, seed=4)
  a = dyn.EINetwork.fixed_prob(3200, 800, seed=2, V0=V0)
  b = dyn.EINetwork(a.n, a.n_exc, indices=a.indices, indptr=a.indptr, V0=V0)
  c = dyn.EINetwork(a.n, a.n_exc, indices=a.indices, indptr=a.indptr, V0=V0)
  ca, _ = a.run(300, method="cluster")
  cb, _ = b.run(300, method="ops")
  cc, _ = c.run(300, method="ops", graph_steps=50)
  assert torch.equal(ca, cb) and torch.equal(ca, cc)
  assert torch.equal(a.V, b.V) and torch.equal(a.V, c.V)


def test_many_networks_of_uneven_sizes(dyn, orc):
  """Networks needing 1, 2, 4 and 16 CTAs run concurrently in one call per cluster size."""
  rng = np.random.default_rng(7)
  sizes = [1000, 2500, 6000, 9000, 15000, 62000]
  nets, states = [], []
  for k, n in enumerate(sizes):
    ne = int(0.8 * n)
    net = dyn.EINetwork.fixed_prob(ne, n - ne, prob=0.02, we=float(rng.uniform(0.3, 1.0)),
                                   wi=float(rng.uniform(3, 10)), seed=10 + k, V0=_v0(n, seed=20 + k))
    nets.append(net)
    states.append(net.state_numpy())
  counts = [torch.zeros(60, dtype=torch.int32, device="cuda") for _ in nets]
  dyn.run_networks(nets, 60, spike_counts=counts)
  for net, st, cnt in zip(nets, states, counts):
    rc, _ = _oracle_run(orc, net, st, 60)
    np.testing.assert_array_equal(cnt.cpu().numpy(), rc)
    np.testing.assert_array_equal(net.V.cpu().numpy(), st["V"])


def test_continue_across_calls(dyn):
  """Two runs of 40 steps equal one run of 80 (state, spikes and time index carried over)."""
  V0 = _v0(4000, seed=5)
  a = dyn.EINetwork.fixed_prob(3200, 800, seed=3, V0=V0)
  b = dyn.EINetwork(a.n, a.n_exc, indices=a.indices, indptr=a.indptr, V0=V0)
  c1, _ = a.run(40)
  c2, _ = a.run(40)
  cb, _ = b.run(80)
  assert torch.equal(torch.cat([c1, c2]), cb) and torch.equal(a.V, b.V)


def _oracle_delayed(orc, net, state, steps, step0=0):
  p = net.params
  op = orc.lif_params(p.V_rest, p.V_th, p.V_reset, p.tau, p.tau_ref, p.R, p.tau_e, p.tau_i, p.E_e, p.E_i, p.input,
                      p.ltc)
  ep, ei, ip, ii = _oracle_split(net)
  return orc.coba_net_run_delayed(op, net.n, net.n_exc, ep, ei, np.float32(net.we), ip, ii, np.float32(net.wi),
                                  state, step0, steps, np.float32(0.1), net.d_e, net.d_i)


@pytest.mark.parametrize("ne,ni,delays", [(3200, 800, (0.5, 0.3)), (3200, 800, (None, 1.2)),
                                           (12000, 3000, (0.2, 0.7)), (3200, 800, (6.4, 6.4))])
def test_delays_cluster_against_oracle(dyn, orc, ne, ni, delays):
  """Synaptic delays on the E and I rows (VarDelay, brainpy/_src/delay.py:334-373): the
  persistent runner, split over two calls, against the oracle's rotating delay buffer."""
  V0 = _v0(ne + ni, seed=8)
  net = dyn.EINetwork.fixed_prob(ne, ni, prob=0.02, seed=5, V0=V0, delay_e=delays[0], delay_i=delays[1])
  assert (net.d_e, net.d_i) == tuple(0 if d is None else int(np.ceil(d / 0.1)) for d in delays)
  state = net.state_numpy()
  c1, _ = net.run(150, method="cluster")
  c2, _ = net.run(250, method="cluster")
  rc = _oracle_delayed(orc, net, state, 400)
  np.testing.assert_array_equal(torch.cat([c1, c2]).cpu().numpy(), rc)
  got = net.state_numpy()
  for k in ("V", "ge", "gi", "t_last", "spike"):
    np.testing.assert_array_equal(got[k], state[k], err_msg=k)
  assert rc.sum() > 500


def test_delays_ops_and_graph_match_cluster(dyn):
  V0 = _v0(4000, seed=9)
  kw = dict(delay_e=0.4, delay_i=0.9)
  a = dyn.EINetwork.fixed_prob(3200, 800, seed=3, V0=V0, **kw)
  b = dyn.EINetwork(a.n, a.n_exc, indices=a.indices, indptr=a.indptr, V0=V0, **kw)
  c = dyn.EINetwork(a.n, a.n_exc, indices=a.indices, indptr=a.indptr, V0=V0, **kw)
  ca, _ = a.run(300, method="cluster")
  cb, _ = b.run(300, method="ops")
  cc, _ = c.run(300, method="ops", graph_steps=40)
  assert torch.equal(ca, cb) and torch.equal(ca, cc)
  assert torch.equal(a.V, b.V) and torch.equal(a.V, c.V)
  assert torch.equal(a.ring, b.ring) and torch.equal(a.ring, c.ring)
  with pytest.raises(ValueError):
    a.run(10, dt=0.05)


def test_spike_ring_reads_as_reference_delay(bplib):
  """The device's spike history (bp_spike_ring_record / bp_spike_ring_read) reads, at every
  step, what the reference's VarDelay reads (tests/golden/consumer.npz, generated by
  executing VarDelay.at / .retrieve / .update of brainpy/_src/delay.py): 8 neurons spike the
  bits of step + 1, so a read decodes to the step it came from (0: nothing recorded yet)."""
  import ctypes
  from golden_util import load
  from brainpy_gb300 import _lib
  L = _lib.lib()
  cons = load("consumer")
  st = _lib.stream_handle()
  for key in [k for k in cons.files if k.startswith("delay|")]:
    _, ring_len, d = key.split("|")
    ring_len, d = int(ring_len[1:]), int(d[1:])
    want = cons[key]
    ring = torch.zeros(ring_len, dtype=torch.int32, device="cuda")  # [ring_len][ceil(8 / 32)] words
    out = torch.empty(8, dtype=torch.uint8, device="cuda")
    for T in range(want.shape[0]):
      _lib.check(L.bp_spike_ring_read(_lib.ptr(ring), ring_len, 8, 0, 8, d, T, None, _lib.ptr(out), st), "ring_read")
      bits = out.cpu().numpy()
      got = int(sum(int(b != 0) << j for j, b in enumerate(bits))) - 1
      assert got == int(want[T]), (key, T, got, int(want[T]))
      sp = torch.tensor([((T + 1) >> j) & 1 for j in range(8)], dtype=torch.uint8, device="cuda")
      _lib.check(L.bp_spike_ring_record(_lib.ptr(sp), 8, _lib.ptr(ring), ring_len, T, None, st), "ring_record")


def _jit_csr(orc, ne, ni, prob, seeds):
  """The four just-in-time projections (E2E, E2I, I2E, I2I; shape (post, pre), pull form) as
  explicit connections from the oracle's generation of the same streams, merged into the
  oracle network's excitatory-row and inhibitory-row CSR matrices over all n post columns."""
  from brainpy_gb300.math.jitconn import conn_len
  clen = conn_len(prob)
  pre_all, post_all = [], []
  for s, (n_post, n_pre, post_off, pre_off) in zip(seeds, ((ne, ne, 0, 0), (ni, ne, ne, 0), (ne, ni, 0, ne),
                                                           (ni, ni, ne, ne))):
    rows, cols, _ = orc.jitconn_connections("homo", 1.0, 0.0, clen, s, n_post, n_pre, True, "gpu")
    post_all.append(rows + post_off)
    pre_all.append(cols + pre_off)
  pre, post = np.concatenate(pre_all), np.concatenate(post_all)
  order = np.argsort(pre, kind="stable")
  pre, post = pre[order], post[order]
  out = []
  for lo, hi in ((0, ne), (ne, ne + ni)):
    sel = (pre >= lo) & (pre < hi)
    ptr = np.concatenate([[0], np.cumsum(np.bincount(pre[sel] - lo, minlength=hi - lo))]).astype(np.int32)
    out += [ptr, np.ascontiguousarray(post[sel].astype(np.int32))]
  return out


def test_jitconn_network_against_oracle(dyn, orc):
  """EINetwork(jitconn=...) -- the four EventJitFPHomoLinear projections (brainpy/_src/dnn/
  linear.py:1044-1280) feeding the COBA outputs (align_post.py:271-275) -- run on the
  per-operator path, host loop and CUDA-graph replay, against the oracle network on the same
  connectivity regenerated by the oracle: spike counts of every step and the final state bit
  for bit (homogeneous weights: exact event counts times w on both sides)."""
  ne, ni, prob, seeds = 1600, 400, 0.05, (11, 12, 13, 14)
  V0 = _v0(ne + ni, seed=21)
  jit = dict(prob=prob, seeds=seeds)
  a = dyn.EINetwork(ne + ni, ne, jitconn=jit, V0=V0)
  b = dyn.EINetwork(ne + ni, ne, jitconn=jit, V0=V0)
  state = a.state_numpy()
  ca, _ = a.run(300, method="ops")
  cb, _ = b.run(300, method="ops", graph_steps=50)
  ep, ei, ip, ii = _jit_csr(orc, ne, ni, prob, seeds)
  p = a.params
  op = orc.lif_params(p.V_rest, p.V_th, p.V_reset, p.tau, p.tau_ref, p.R, p.tau_e, p.tau_i, p.E_e, p.E_i, p.input,
                      p.ltc)
  rc, _ = orc.coba_net_run(op, a.n, ne, ep, ei, np.float32(a.we), ip, ii, np.float32(a.wi), state, 0, 300,
                           np.float32(0.1), count_mode=True)
  np.testing.assert_array_equal(ca.cpu().numpy(), rc)
  np.testing.assert_array_equal(cb.cpu().numpy(), rc)
  for net in (a, b):
    got = net.state_numpy()
    for k in ("V", "ge", "gi", "t_last", "spike"):
      np.testing.assert_array_equal(got[k], state[k], err_msg=k)
  assert rc.sum() > 300  # the network is active


@pytest.mark.parametrize("index_dtype", [None, torch.int64])
def test_materialized_jitconn_network(dyn, orc, index_dtype):
  """EINetwork.materialize(): the four pull projections' connections stored as one
  presynaptic-row CSR (bp_jitconn_csr) are the oracle's regeneration of the same streams, row
  by row, and the stored network spikes as the just-in-time one does, bit for bit: its
  per-operator path, the cluster runner and the whole-GPU runner against the just-in-time
  network's per-operator path (exact event counts times w on every path)."""
  ne, ni, prob, seeds = 1600, 400, 0.05, (11, 12, 13, 14)
  n = ne + ni
  V0 = _v0(n, seed=21)
  a = dyn.EINetwork(n, ne, jitconn=dict(prob=prob, seeds=seeds), V0=V0)
  m = a.materialize(index_dtype=index_dtype)
  assert m.jitconn is None and m.indices.dtype == (index_dtype or torch.int32)
  ep, ei, ip, ii = _jit_csr(orc, ne, ni, prob, seeds)
  want_ptr = np.concatenate([ep.astype(np.int64), ip[1:].astype(np.int64) + int(ep[-1])])
  want_ind = np.concatenate([ei, ii]).astype(np.int64)
  ptr = m.indptr.cpu().numpy().astype(np.int64)
  ind = m.indices.cpu().numpy().astype(np.int64)
  np.testing.assert_array_equal(ptr, want_ptr)
  rows = np.repeat(np.arange(n), np.diff(ptr))
  got = np.lexsort((ind, rows))
  want = np.lexsort((want_ind, rows))
  np.testing.assert_array_equal(ind[got], want_ind[want])  # the same posts in every row
  ca, _ = a.run(300, method="ops")
  recs = m.tune_ops()  # the chosen kernels give the same products
  assert len(recs) == 2 and all("choice" in r for r in recs)
  runs = [m.run(300, method="ops")[0]]
  for method in ("cluster", "grid"):
    x = a.materialize(index_dtype=index_dtype)
    x.reset_state(torch.as_tensor(V0, device="cuda"), torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda"),
                  torch.full((n,), -1e7, device="cuda"), torch.zeros(n, dtype=torch.bool, device="cuda"))
    runs.append(x.run(300, method=method)[0])
  for c in runs:
    np.testing.assert_array_equal(c.cpu().numpy(), ca.cpu().numpy())
  sa, sm = a.state_numpy(), m.state_numpy()
  for k in ("V", "ge", "gi", "t_last", "spike"):
    np.testing.assert_array_equal(sm[k], sa[k], err_msg=k)
  assert int(ca.sum()) > 300  # the network is active


def test_autotuned_tiles_and_concurrent_launches_match(dyn):
  """Networks of several size classes: tiles chosen by autotune_net_tiles and the launches of
  the cluster sizes run concurrently give the same spike counts and state, bit for bit, as
  the default tiles with the launches in stream order; a cached choice is applied without
  timing."""
  from brainpy_gb300 import tuning
  sizes = [1500, 3000, 6000, 20000, 45000]
  def make():
    return [dyn.EINetwork.fixed_prob(int(0.8 * n), n - int(0.8 * n), seed=30 + k, V0=_v0(n, seed=40 + k))
            for k, n in enumerate(sizes)]
  a, b = make(), make()
  ca = [torch.zeros(300, dtype=torch.int32, device="cuda") for _ in a]
  cb = [torch.zeros(300, dtype=torch.int32, device="cuda") for _ in b]
  dyn.run_networks(a, 300, spike_counts=ca, concurrent=False)
  cache = tuning.TuneCache()
  rec = dyn.autotune_net_tiles(b, steps=40, cache=cache)
  assert rec and all(r["choice"] in (1024, 2048, 4096) for r in rec.values())
  assert all(x.net_tile == rec[dyn.size_class(x.n)]["choice"] for x in b)
  dyn.run_networks(b, 300, spike_counts=cb)
  for x, y, c1, c2 in zip(a, b, ca, cb):
    assert torch.equal(c1, c2) and torch.equal(x.V, y.V) and torch.equal(x.t_last, y.t_last)
    assert int(c1.sum()) > 0
  # the same classes again: the cached records are applied, nothing is timed
  c = make()
  rec2 = dyn.autotune_net_tiles(c, steps=40, cache=cache)
  assert {k: v["choice"] for k, v in rec2.items()} == {k: v["choice"] for k, v in rec.items()}


def test_batch_graph_replays_continue(dyn):
  """NetBatch: the launches captured once as a CUDA graph and replayed twice (new spike-count
  outputs and a step limit on the second replay) give what two plain batched runs give."""
  sizes = [2000, 5000, 12000]
  def make():
    return [dyn.EINetwork.fixed_prob(int(0.8 * n), n - int(0.8 * n), seed=50 + k, V0=_v0(n, seed=60 + k))
            for k, n in enumerate(sizes)]
  a, b = make(), make()
  lim = [0, 90, 0]
  ca = [[torch.zeros(120, dtype=torch.int32, device="cuda") for _ in a] for _ in range(2)]
  cb = [[torch.zeros(120, dtype=torch.int32, device="cuda") for _ in b] for _ in range(2)]
  dyn.run_networks(a, 120, spike_counts=ca[0])
  dyn.run_networks(a, 120, spike_counts=ca[1], step_limits=lim)
  batch = dyn.NetBatch(b)
  batch.capture(120)
  batch.replay(spike_counts=cb[0])
  batch.replay(spike_counts=cb[1], step_limits=lim)
  for r in range(2):
    for x, y in zip(ca[r], cb[r]):
      assert torch.equal(x, y)
  for x, y in zip(a, b):
    assert x.t_step == y.t_step and torch.equal(x.V, y.V) and torch.equal(x.spike, y.spike)
  assert [x.t_step for x in b] == [240, 210, 240]


def _big_net(dyn, n, prob, seed, V0seed):
  ne = int(0.8 * n)
  s = 80.0 / (prob * n)  # COBA's total drive at this fan-out
  return dyn.EINetwork.fixed_prob(ne, n - ne, prob=prob, we=0.6 * s, wi=6.7 * s, seed=seed, V0=_v0(n, seed=V0seed))


def test_grid_runner_against_oracle(dyn, orc):
  """A network larger than one cluster (100,000 neurons, fan-out 1000) in one persistent launch
  over the GPU: spike counts of every step, the V trace of the first 50 steps and the final
  state bit-exact against the oracle network; the barrier waits all ended."""
  net = _big_net(dyn, 100_000, 0.01, seed=7, V0seed=8)
  assert not net.fits_cluster() and net.grid_eligible()
  state = net.state_numpy()
  counts, trace = net.run(300, v_trace_steps=50)  # method "cluster" takes the grid runner here
  assert net.grid_error() == 0
  from brainpy_gb300 import _lib
  print("grid runner cooperative launch:", _lib.lib().bp_net_grid_cooperative())
  rc, rtrace = _oracle_run(orc, net, state, 300, trace_steps=50)
  np.testing.assert_array_equal(counts.cpu().numpy(), rc)
  np.testing.assert_array_equal(trace.cpu().numpy(), rtrace)
  got = net.state_numpy()
  for k in ("V", "ge", "gi", "t_last", "spike"):
    np.testing.assert_array_equal(got[k], state[k], err_msg=k)
  assert rc.sum() > 10_000


def test_grid_runner_matches_ops_path_across_calls(dyn):
  """300,000 neurons: two grid runs of 100 steps equal one per-operator run of 200 steps (graph
  replay), bit for bit."""
  a = _big_net(dyn, 300_000, 0.001, seed=9, V0seed=10)
  b = dyn.EINetwork(a.n, a.n_exc, indices=a.indices, indptr=a.indptr, we=a.we, wi=a.wi, V0=a.V.clone())
  c1, _ = a.run(100, method="grid")
  c2, _ = a.run(100, method="grid")
  cb, _ = b.run(200, method="ops", graph_steps=50)
  assert a.grid_error() == 0
  assert torch.equal(torch.cat([c1, c2]), cb)
  for k in ("V", "ge", "gi", "t_last", "spike"):
    assert torch.equal(getattr(a, k), getattr(b, k)), k
  assert int(cb.sum()) > 1000 and a.t_step == 200


@pytest.mark.parametrize("n,n_exc", [(70_001, 56_000), (65_600, 65_600)])
def test_grid_runner_odd_sizes(dyn, n, n_exc):
  """Sizes whose last tile and last CTA are partly empty, and a network with no inhibitory
  neuron: the grid runner equals the per-operator path, spike counts and state."""
  fan = 300
  ind_e, _ = dyn.fixed_prob_csr(n, n, fan, seed=n % 97)
  ptr = torch.arange(n + 1, device="cuda", dtype=torch.int64) * fan
  s = 80.0 / fan
  V0 = _v0(n, seed=n % 89)
  a = dyn.EINetwork(n, n_exc, indices=ind_e, indptr=ptr.to(torch.int32), we=0.6 * s, wi=6.7 * s, V0=V0)
  b = dyn.EINetwork(n, n_exc, indices=ind_e, indptr=ptr.to(torch.int32), we=0.6 * s, wi=6.7 * s, V0=V0)
  assert a.grid_eligible()
  ca, _ = a.run(150, method="grid")
  cb, _ = b.run(150, method="ops")
  assert a.grid_error() == 0
  assert torch.equal(ca, cb) and int(ca.sum()) > 0
  for k in ("V", "ge", "gi", "t_last", "spike"):
    assert torch.equal(getattr(a, k), getattr(b, k)), k


def test_grid_runner_delays_match_ops_path(dyn):
  """Synaptic delays on the grid runner (spike history in global memory, each CTA its own
  words): 120,000 neurons, excitatory rows delayed 0.4 ms and inhibitory rows 0.9 ms, in two
  runs of 90 steps, equal to one per-operator run of 180 steps: spike counts, state and the
  history ring, bit for bit."""
  n = 120_000
  ne = int(0.8 * n)
  s = 80.0 / (0.005 * n)
  kw = dict(delay_e=0.4, delay_i=0.9)
  a = dyn.EINetwork.fixed_prob(ne, n - ne, prob=0.005, we=0.6 * s, wi=6.7 * s, seed=17, V0=_v0(n, seed=18), **kw)
  b = dyn.EINetwork(a.n, a.n_exc, indices=a.indices, indptr=a.indptr, we=a.we, wi=a.wi, V0=a.V.clone(), **kw)
  assert a.grid_eligible() and a.ring is not None
  c1, _ = a.run(90, method="grid")
  c2, _ = a.run(90, method="grid")
  cb, _ = b.run(180, method="ops")
  assert a.grid_error() == 0
  assert torch.equal(torch.cat([c1, c2]), cb) and int(cb.sum()) > 0
  for k in ("V", "ge", "gi", "t_last", "spike", "ring"):
    assert torch.equal(getattr(a, k), getattr(b, k)), k


@pytest.mark.parametrize("n", [50_000, 400_000])
def test_grid_runner_jitconn_push_matches_ops_path(dyn, n):
  """A just-in-time network in the push form (outdim_parallel=False, the served jitconn jobs)
  on the whole-GPU runner, in two runs, equal to the per-operator path (event_mv_prob_homo
  push per projection) bit for bit: spike counts of every step and the final state."""
  ne = int(0.8 * n)
  fan = 1000
  jit = dict(prob=fan / n, seeds=(21, 22, 23, 24), outdim_parallel=False)
  s = 80.0 / fan
  V0 = _v0(n, seed=31)
  a = dyn.EINetwork(n, ne, jitconn=jit, we=0.6 * s, wi=6.7 * s, V0=V0)
  b = dyn.EINetwork(n, ne, jitconn=jit, we=0.6 * s, wi=6.7 * s, V0=V0)
  assert a.grid_eligible() and not a.fits_cluster()
  c1, _ = a.run(60)  # method "cluster" takes the whole-GPU runner for this network
  c2, _ = a.run(60, method="grid")
  cb, _ = b.run(120, method="ops")
  assert a.grid_error() == 0
  assert torch.equal(torch.cat([c1, c2]), cb) and int(cb.sum()) > 0
  for k in ("V", "ge", "gi", "t_last", "spike"):
    assert torch.equal(getattr(a, k), getattr(b, k)), k
