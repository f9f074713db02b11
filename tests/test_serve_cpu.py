"""Host logic of the serving loop without a GPU: FIFO admission under the HBM budget (no
overtaking; a job larger than the budget still runs when nothing else is admitted), retirement
returning the memory, and the job-memory estimate's monotonicity.  The device work is stubbed:
building a job returns a placeholder and its spike counts live on the CPU."""
import numpy as np
import pytest
import torch

import brainpy_gb300.serve as serve


def _server(monkeypatch, budget):
  monkeypatch.setattr(serve, "build_job", lambda job, device: object())
  srv = serve.Server(hbm_budget_bytes=budget, side_streams=0, device=torch.device("cpu"), build_thread=False)
  srv._fits_cluster = lambda job: True  # no side stream needed for a stubbed job
  return srv


def _jobs(sizes, arrivals=None):
  arrivals = arrivals or [0.0] * len(sizes)
  return [serve.Job(k, n, "csr", 1.0, 0.6, 6.7, arrival=a, seed=k) for k, (n, a) in enumerate(zip(sizes, arrivals))]


def _finish(srv, job):
  job.steps_done = job.steps_total
  srv._retire()


def test_job_memory_grows_with_size():
  prev = 0
  for n in (1000, 4000, 20000, 65536, 100000, 1_000_000):
    m = serve.job_memory(serve.Job(0, n, "csr", 100.0, 0.6, 6.7))
    assert m > prev
    prev = m
  # just-in-time connectivity holds no synapse arrays
  assert serve.job_memory(serve.Job(0, 100000, "jitconn", 100.0, 0.6, 6.7)) < \
      serve.job_memory(serve.Job(0, 100000, "csr", 100.0, 0.6, 6.7))


def test_fifo_admission_under_budget(monkeypatch):
  jobs = _jobs([20000, 20000, 20000, 3000])
  need = serve.job_memory(jobs[0])
  small = serve.job_memory(jobs[3])
  assert small < 0.5 * need
  srv = _server(monkeypatch, budget=2.5 * need)
  for j in jobs:
    srv.submit(j)
  srv.t0 = 0.0
  srv.now = lambda: 1.0
  srv._admit()
  # two large jobs fit; the third would not, and the small job behind it waits (no overtaking)
  assert [j.jid for j in srv.active] == [0, 1]
  assert srv.used == 2 * need
  assert [j.jid for j in srv.queue] == [2, 3]
  # retiring one job frees its memory: the large job at the head enters, then the small one
  _finish(srv, srv.active[0])
  assert srv.used == need
  srv._admit()
  assert [j.jid for j in srv.active] == [1, 2, 3]
  assert srv.used == 2 * need + small
  assert srv.queue == []
  assert [j.jid for j in srv.done] == [0]
  assert srv.done[0].result is not None and srv.done[0].result.shape == (srv.done[0].steps_total,)


def test_oversized_job_runs_alone(monkeypatch):
  jobs = _jobs([50000, 3000])
  srv = _server(monkeypatch, budget=0.5 * serve.job_memory(jobs[0]))
  for j in jobs:
    srv.submit(j)
  srv.t0 = 0.0
  srv.now = lambda: 1.0
  srv._admit()
  # nothing is admitted yet, so the oversized head of the queue runs on its own
  assert [j.jid for j in srv.active] == [0]
  assert [j.jid for j in srv.queue] == [1]
  _finish(srv, srv.active[0])
  srv._admit()
  assert [j.jid for j in srv.active] == [1]


def test_arrivals_gate_admission(monkeypatch):
  jobs = _jobs([3000, 3000, 3000], arrivals=[0.5, 0.0, 2.0])
  srv = _server(monkeypatch, budget=1e15)
  for j in jobs:
    srv.submit(j)
  assert [j.arrival for j in srv.queue] == sorted(j.arrival for j in jobs)
  srv.t0 = 0.0
  srv.now = lambda: 1.0
  srv._admit()
  assert sorted(j.jid for j in srv.active) == [0, 1]
  assert [j.jid for j in srv.queue] == [2]
  assert all(j.admitted_at == 1.0 for j in srv.active)
  assert all(np.all(j.counts.numpy() == 0) for j in srv.active)


@pytest.mark.parametrize("n_jobs", [1, 30])
def test_poisson_jobs_stream(n_jobs):
  jobs = serve.poisson_jobs(n_jobs, seed=3)
  assert len(jobs) == n_jobs
  t = [j.arrival for j in jobs]
  assert t == sorted(t) and t[0] > 0
  assert all(4000 <= j.n <= 1_000_000 and 100.0 <= j.duration_ms <= 2000.0 for j in jobs)
  assert all(j.conn in ("csr", "jitconn") for j in jobs)
  again = serve.poisson_jobs(n_jobs, seed=3)
  assert [(j.n, j.conn, j.arrival) for j in again] == [(j.n, j.conn, j.arrival) for j in jobs]


def test_builds_run_off_the_scheduling_thread(monkeypatch):
  """Admitted jobs are built by the worker thread; they join the stepping set on a later
  admission pass once their build has finished, in admission order, and nothing is lost."""
  import threading
  gate = threading.Event()

  def slow_build(job, device):
    gate.wait(10.0)
    return object()

  monkeypatch.setattr(serve, "build_job", slow_build)
  srv = serve.Server(hbm_budget_bytes=1e15, side_streams=0, device=torch.device("cpu"))
  srv._fits_cluster = lambda job: True
  try:
    for j in _jobs([3000, 4000, 5000]):
      srv.submit(j)
    srv.t0 = 0.0
    srv.now = lambda: 1.0
    srv._admit()
    # admitted (memory reserved) but still building: the scheduling thread did not wait
    assert srv.active == [] and [j.jid for j, _ in srv.building] == [0, 1, 2]
    assert srv.used == sum(serve.job_memory(j) for j, _ in srv.building)
    gate.set()
    for _, fut in list(srv.building):
      fut.result(timeout=10.0)
    srv._admit()
    assert [j.jid for j in srv.active] == [0, 1, 2] and srv.building == []
    assert all(j.built_by.startswith("bp-serve-build") for j in srv.active)
  finally:
    gate.set()
    srv.close()
