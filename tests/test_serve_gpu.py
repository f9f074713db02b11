"""The serving loop: every job's result equals the same job run alone, jobs wait for HBM
budget, and all jobs complete."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve(bplib):
  import brainpy_gb300.serve as s
  return s


def _alone(serve, job, dev, chunk=100, graph_steps=50):
  net = serve.build_job(job, dev)
  steps = int(round(job.duration_ms / 0.1))
  fits = job.conn == "csr" and job.n <= 16 * 4096
  counts = torch.zeros(steps, dtype=torch.int32, device=dev)
  if fits:
    net.run(steps, spike_counts=counts)
  else:
    done = 0
    while done < steps:  # the server's chunking: graphs of 50 steps inside chunks of 100
      k = min(chunk, steps - done)
      net.run(k, method="ops", spike_counts=counts[done:done + k], graph_steps=graph_steps if k >= graph_steps else 0)
      done += k
  return counts.cpu().numpy()


def _mix(serve):
  J = serve.Job
  return [J(0, 3000, "csr", 12.0, 0.6, 6.7, arrival=0.0, seed=1),
          J(1, 9000, "csr", 20.0, 0.5, 5.0, arrival=0.0, seed=2),
          J(2, 70000, "csr", 15.0, 0.7, 6.0, arrival=0.01, seed=3, fanout=300),
          J(3, 5000, "jitconn", 13.0, 0.6, 6.7, arrival=0.0, seed=4, fanout=200),
          J(4, 30000, "jitconn", 7.3, 0.4, 8.0, arrival=0.02, seed=5, fanout=500),
          J(5, 2000, "csr", 3.1, 0.9, 9.0, arrival=0.03, seed=6)]


def test_results_equal_alone(serve):
  dev = torch.device("cuda")
  jobs = _mix(serve)
  srv = serve.Server(hbm_budget_bytes=50e9)
  for j in jobs:
    srv.submit(j)
  srv.run(max_seconds=120)
  assert len(srv.done) == len(jobs)
  for j in sorted(srv.done, key=lambda x: x.jid):
    ref = _alone(serve, j, dev)
    np.testing.assert_array_equal(j.result, ref, err_msg=f"job {j.jid} ({j.conn}, n={j.n})")
    assert j.result.sum() > 0 and j.latency > 0
    assert j.built_by.startswith("bp-serve-build")  # built on the worker thread
  srv.close()


def test_budget_admission(serve):
  dev = torch.device("cuda")
  J = serve.Job
  jobs = [J(k, 20000, "csr", 5.0, 0.6, 6.7, arrival=0.0, seed=20 + k) for k in range(3)]
  need = serve.job_memory(jobs[0])
  srv = serve.Server(hbm_budget_bytes=1.5 * need)  # one job at a time
  for j in jobs:
    srv.submit(j)
  srv.run(max_seconds=120)
  done = sorted(srv.done, key=lambda x: x.jid)
  assert len(done) == 3
  for a, b in zip(done, done[1:]):
    assert b.admitted_at >= a.finished_at
  for j in done:
    np.testing.assert_array_equal(j.result, _alone(serve, j, dev))
