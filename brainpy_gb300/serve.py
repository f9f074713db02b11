"""Continuous-batching server for spiking-network simulation jobs.

A job is one E/I COBA network (n neurons, 80/20, LifRefLTC) simulated for a given duration.
Its connectivity is either CSR (2 % FixedProb, fan-out capped) or just-in-time with a fixed
fan-out (event_mv_prob_homo, outdim_parallel=False: the connections of every spiking neuron
are regenerated from its LFSR88 streams).

The loop:
  * admission: arrived jobs enter in FIFO order while their estimated device memory fits the
    HBM budget; state and connectivity then stay resident on the device until the job ends;
  * building: an admitted job's network (FixedProb generation, plan, counters, workspaces) is
    built on a worker thread into its own CUDA stream, so a burst of arrivals does not stall
    the jobs already stepping; the job joins the stepping set once its build has finished on
    the host, its streams ordered after the build by a CUDA event;
  * every iteration advances all admitted jobs by one chunk of steps: CSR jobs that fit one
    thread-block cluster (n <= 16 x 4096) run together in persistent cluster launches (one per
    cluster size, every network at its own time index and step limit); larger CSR jobs run
    one whole-GPU persistent launch each (bp_net_run_grid); the jitconn jobs run their
    per-operator steps from per-job CUDA graphs spread over side streams, so their kernels
    overlap on the device;
  * finished jobs are retired (spike counts copied to the host, memory released) and their
    latency (arrival to result on the host) recorded.
A job's result does not depend on what it shares the device with: every path is deterministic
(integer event counts; homogeneous-weight atomics add equal values).
"""
import math
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import List, Optional

import numpy as np
import torch

from . import _lib
from . import dyn


@dataclass
class Job:
  jid: int
  n: int
  conn: str  # "csr" or "jitconn"
  duration_ms: float
  we: float
  wi: float
  arrival: float = 0.0  # seconds after the server starts
  seed: int = 0
  fanout: int = 1000
  # runtime
  steps_total: int = 0
  steps_done: int = 0
  net: Optional[dyn.EINetwork] = None
  counts: Optional[torch.Tensor] = None
  mem: int = 0
  admitted_at: float = -1.0
  finished_at: float = -1.0
  result: Optional[np.ndarray] = None
  stream: Optional[torch.cuda.Stream] = None
  built_by: str = ""  # the host thread that built the job
  path: str = ""      # "cluster", "grid" or "ops": how the job steps

  @property
  def latency(self):
    return self.finished_at - self.arrival


def job_memory(job: Job) -> int:
  """Device bytes a job holds while admitted: its state (V, ge, gi, t_last in float32 and the
  spike byte of every neuron, one spike count per step); for a CSR job also the int32 indices
  and indptr, one tiled plan (segment offsets, 4 bytes per row and tile boundary, and 2 bytes
  per padded entry: the cluster runner's plan of 4096-column tiles, or the per-operator path's
  two projection plans, which together cover the same rows) and the per-operator path's event
  workspace (the active-row lists of the rows); a jitconn job stores no matrix."""
  n = job.n
  state = n * (4 * 4 + 1) + 4 * int(job.duration_ms / 0.1 + 1)
  if job.conn == "jitconn":
    return state + 8 * n
  k = min(int(0.02 * n), job.fanout)
  nnz = n * k
  tiles = math.ceil(n / 4096) if n <= 16 * 4096 else max(1, math.ceil(n / 27840))
  plan = 4 * n * (tiles + 1) + 2 * (nnz + (8 * tiles + 8) * n + 8)
  lists = 4 * (math.ceil(n / 4096) * 4096 + math.ceil(n / 4096)) + 1024
  return state + 4 * nnz + 4 * (n + 1) + plan + lists


def build_job(job: Job, device) -> dyn.EINetwork:
  n = job.n
  ne = int(0.8 * n)
  rng = np.random.default_rng(job.seed)
  V0 = rng.normal(-55.0, 5.0, n).astype(np.float32)
  if job.conn == "jitconn":
    # fan-out `fanout` per presynaptic neuron: p = fanout / n_post per projection; COBA weights
    # scaled by 80 / fanout keep the example's total drive
    s = 80.0 / job.fanout
    return dyn.EINetwork(n, ne, jitconn=dict(prob=min(1.0, job.fanout / n), seeds=tuple(job.seed * 4 + k for k in range(4)),
                                             outdim_parallel=False),
                         we=job.we * s, wi=job.wi * s, device=device, V0=V0)
  prob = min(0.02, job.fanout / n)
  return dyn.EINetwork.fixed_prob(ne, n - ne, prob=prob, we=job.we, wi=job.wi, seed=job.seed, device=device, V0=V0)


class Server:
  def __init__(self, hbm_budget_bytes: float = 150e9, chunk_steps: int = 100, dt: float = 0.1, side_streams: int = 4,
               graph_steps: int = 50, device=None, build_thread: bool = True):
    self.budget = float(hbm_budget_bytes)
    self.chunk = int(chunk_steps)
    self.dt = float(dt)
    self.graph_steps = int(graph_steps)
    self.device = device or torch.device("cuda", torch.cuda.current_device())
    self.streams = [torch.cuda.Stream(device=self.device) for _ in range(side_streams)]
    self.build_stream = torch.cuda.Stream(device=self.device) if self.device.type == "cuda" else None
    self._pool = ThreadPoolExecutor(max_workers=1, thread_name_prefix="bp-serve-build") if build_thread else None
    self.building = []  # (job, future of its build event), in admission order
    self.queue: List[Job] = []
    self.active: List[Job] = []
    self.done: List[Job] = []
    self.used = 0
    self.t0 = None
    self.events = 0

  def now(self):
    return time.perf_counter() - self.t0

  def submit(self, job: Job):
    job.steps_total = int(round(job.duration_ms / self.dt))
    self.queue.append(job)
    self.queue.sort(key=lambda j: j.arrival)

  # ---- scheduling -------------------------------------------------------------------
  def _admit(self):
    t = self.now()
    while self.queue and self.queue[0].arrival <= t:
      job = self.queue[0]
      need = job_memory(job)
      if self.used + need > self.budget and (self.active or self.building):
        break  # wait for memory to free up (FIFO: no overtaking)
      self.queue.pop(0)
      job.mem = need
      self.used += need
      job.admitted_at = self.now()
      if self._pool is not None:
        self.building.append((job, self._pool.submit(self._build, job)))
      else:
        self._activate(job, self._build(job))
    # jobs whose build has finished join the stepping set (a failed build raises here)
    pending = []
    for job, fut in self.building:
      if fut.done():
        self._activate(job, fut.result())
      else:
        pending.append((job, fut))
    self.building = pending

  def _build(self, job):
    """The job's network, spike counters and the connectivity structures its path reads (the
    cluster runner's plan, or the per-operator path's projection plans and workspaces), all
    on the build stream.  Runs on the worker thread; returns a CUDA event recorded after the
    last of that work."""
    job.built_by = threading.current_thread().name
    if self.build_stream is None:  # host-only use (no device work to order)
      job.net = build_job(job, self.device)
      job.counts = torch.zeros(job.steps_total, dtype=torch.int32, device=self.device)
      job.path = "cluster" if self._fits_cluster(job) else "ops"
      return None
    torch.cuda.set_device(self.device)
    with torch.cuda.stream(self.build_stream):
      job.net = build_job(job, self.device)
      job.counts = torch.zeros(job.steps_total, dtype=torch.int32, device=self.device)
      if self._fits_cluster(job):
        job.path = "cluster"
        job.net._cluster_plan()
      elif job.conn == "csr" and job.net.grid_eligible():
        # jitconn jobs stay on their per-operator graphs: those overlap with the other jobs'
        # kernels on side streams, where a whole-GPU launch holds every SM while it spins
        job.path = "grid"
        job.net._grid_state()
      else:
        job.path = "ops"
        if job.conn == "csr":
          job.net._csr_ops()
      ev = torch.cuda.Event()
      ev.record(self.build_stream)
    return ev

  def _activate(self, job, built):
    """Orders the job's stepping stream after its build and adds it to the stepping set."""
    if built is None:
      pass
    elif job.path in ("cluster", "grid"):
      torch.cuda.current_stream(self.device).wait_event(built)
    else:
      job.stream = self.streams[job.jid % len(self.streams)]
      job.stream.wait_event(built)
    self.active.append(job)

  def _fits_cluster(self, job):
    return job.conn == "csr" and job.n <= _lib.lib().bp_net_max_tiles() * _lib.lib().bp_net_tile_width()

  def _advance(self):
    cl = [j for j in self.active if j.path == "cluster"]
    if cl:
      limits = [min(self.chunk, j.steps_total - j.steps_done) for j in cl]
      outs = [j.counts[j.steps_done:] for j in cl]
      dyn.run_networks([j.net for j in cl], self.chunk, self.dt, spike_counts=outs, step_limits=limits)
      for j, k in zip(cl, limits):
        j.steps_done += k
    for j in self.active:
      if j.path != "grid":
        continue
      # one whole-GPU persistent launch per job and chunk, in turn on the current stream (each
      # holds a cluster on every SM it uses while it runs)
      k = min(self.chunk, j.steps_total - j.steps_done)
      j.net.run(k, self.dt, method="grid", spike_counts=j.counts[j.steps_done:j.steps_done + k])
      j.steps_done += k
    for j in self.active:
      if j.path != "ops":
        continue
      k = min(self.chunk, j.steps_total - j.steps_done)
      with torch.cuda.stream(j.stream):
        g = self.graph_steps if k >= self.graph_steps else 0
        j.net.run(k, self.dt, method="ops", spike_counts=j.counts[j.steps_done:j.steps_done + k], graph_steps=g)
      j.steps_done += k

  def _retire(self):
    finished = [j for j in self.active if j.steps_done >= j.steps_total]
    if not finished:
      return
    for j in finished:
      if j.stream is not None:
        torch.cuda.current_stream(self.device).wait_stream(j.stream)
      j.result = j.counts.cpu().numpy()  # the job's result on the host
      if j.path == "grid" and j.net.grid_error():
        raise RuntimeError(f"job {j.jid}: a grid-barrier wait of the whole-GPU runner ran out")
      j.finished_at = self.now()
      self.events += int(j.result.sum()) * self._fanout(j)
      self.active.remove(j)
      self.used -= j.mem
      j.net = None
      j.counts = None
      self.done.append(j)

  @staticmethod
  def _fanout(j):
    return min(int(0.02 * j.n), j.fanout) if j.conn == "csr" else j.fanout

  def run(self, max_seconds: float = 1e9):
    """Serves every submitted job; returns wall seconds."""
    self.t0 = time.perf_counter()
    while (self.queue or self.active or self.building) and self.now() < max_seconds:
      self._admit()
      if not self.active:
        if self.building:
          time.sleep(0.0005)  # a build in flight: wait for it on the host
        elif self.queue:
          time.sleep(max(0.0, min(0.01, self.queue[0].arrival - self.now())))
        continue
      self._advance()
      self._retire()
    for _, fut in self.building:  # a time limit hit with builds in flight: let them finish
      fut.result()
    torch.cuda.synchronize(self.device)
    return self.now()

  def close(self):
    """Stops the build thread."""
    if self._pool is not None:
      self._pool.shutdown(wait=True)
      self._pool = None


def poisson_jobs(n_jobs, rate_hz=50.0, n_min=4000, n_max=1_000_000, dur_ms=(100.0, 2000.0), seed=0,
                 jitconn_frac=0.5):
  """Job stream: Poisson arrivals, sizes log-uniform, durations uniform, COBA weight draws."""
  rng = np.random.default_rng(seed)
  t = np.cumsum(rng.exponential(1.0 / rate_hz, n_jobs))
  jobs = []
  for k in range(n_jobs):
    n = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
    jobs.append(Job(jid=k, n=n, conn="jitconn" if rng.random() < jitconn_frac else "csr",
                    duration_ms=float(rng.uniform(*dur_ms)), we=float(rng.uniform(0.3, 1.0)),
                    wi=float(rng.uniform(3.0, 10.0)), arrival=float(t[k]), seed=1000 + k))
  return jobs


def bench(args):
  """Serving loop on a bounded sample of the job stream (sizes 4k-1M log-uniform, durations
  100-2000 ms, Poisson 50 jobs/s, HBM budget 150 GB)."""
  n_jobs = args.nets if args.nets != 256 else 60
  # warm-up session (a server in service is warm): a few short jobs of every kind and size class
  warm = Server(hbm_budget_bytes=150e9)
  for k, (n, conn) in enumerate([(5000, "csr"), (200_000, "csr"), (5000, "jitconn"), (200_000, "jitconn")]):
    warm.submit(Job(jid=k, n=n, conn=conn, duration_ms=20.0, we=0.6, wi=6.7, arrival=0.0, seed=7 + k))
  warm.run()
  warm.close()
  del warm
  torch.cuda.synchronize()
  jobs = poisson_jobs(n_jobs)
  srv = Server(hbm_budget_bytes=150e9)
  for j in jobs:
    srv.submit(j)
  wall = srv.run()
  srv.close()
  lat = np.array([j.latency for j in srv.done])
  steps = sum(j.steps_total for j in srv.done)
  # the plain per-network path on the same jobs: one job at a time, one kernel per operator per
  # step from a host loop, a bounded number of steps per job (after one warm-up step); every
  # served job's per-step time, weighted by the job's length as in the served run
  k_plain = 20
  sample = poisson_jobs(n_jobs)
  plain_steps, plain_t = 0, 0.0
  for job in sample:
    net = build_job(job, srv.device)
    net.run(1, method="ops")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net.run(k_plain, method="ops")
    torch.cuda.synchronize()
    per_step = (time.perf_counter() - t0) / k_plain
    n_steps = int(round(job.duration_ms / srv.dt))
    plain_t += per_step * n_steps
    plain_steps += n_steps
    del net
  torch.cuda.empty_cache()
  plain = plain_steps / plain_t
  return {"metric": "served job latency p50 (COBA jobs, continuous batching)", "value": float(np.percentile(lat, 50)),
          "unit": "s", "n_gpus": 1, "steps": steps, "warmup": 0, "ms_per_step": None, "higher_is_better": False,
          "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
          "config": {"workload": f"{n_jobs} jobs, Poisson 50/s, N~logU[4k,1M], 50% CSR 2% (fan-out<=1000) / 50% "
                                 "jitconn fan-out 1000, durations U[100,2000] ms, HBM budget 150 GB"},
          "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
          "jobs_done": len(srv.done), "wall_s": wall, "synaptic_events_per_s": srv.events / wall,
          "network_steps_per_s": steps / wall,
          "plain_per_network_path": {"value": plain, "unit": "network-steps/s",
                                     "sample": f"all {len(sample)} jobs of the stream, one at a time, per-operator "
                                               f"kernels from a host loop; {k_plain} steps timed per job, "
                                               "weighted by the job's length"},
          "speedup_vs_plain": (steps / wall) / plain}
