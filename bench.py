"""Benchmark: event-driven synaptic propagation, event.csrmv transpose=True.

Workload (the operator sweep's headline point): square CSR, N = 1e6 neurons, fan-out
K = 1000 (1e9 synapses, int32 indices), homogeneous float32 weight, bool spike vectors
with a 2 % event rate.  One step = one event.csrmv call on a fresh spike vector
(8 vectors rotate, 640 MB of active rows in total) with L2 flushed (256 MB write)
between timed steps.  Metric: synaptic events/s = (active rows x K) / step time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the reference's CPU implementation of the same operator (its
Numba transpose loop, restated in C because numba/jax are not installable here) on the
host cores, on the same workload.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "synaptic events/s (event.csrmv transpose, N=1e6, fan-out 1000, 2% events)"
UNIT = "events/s"


def parse():
  ap = argparse.ArgumentParser()
  ap.add_argument("--gpus", type=int, default=1)
  ap.add_argument("--steps", type=int, default=50)
  ap.add_argument("--warmup", type=int, default=5)
  ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
  ap.add_argument("--n", type=int, default=1_000_000)
  ap.add_argument("--fanout", type=int, default=1000)
  ap.add_argument("--rate", type=float, default=0.02)
  ap.add_argument("--weights", default="homo", choices=["homo", "heter"])
  ap.add_argument("--no-cpu-baseline", action="store_true")
  ap.add_argument("--cpu-seconds", type=float, default=12.0)
  ap.add_argument("--workload", default="event_csrmv",
                  choices=["event_csrmv", "coba", "batched", "jitconn_net", "serve", "sweep", "vmap", "stdp",
                           "sparse_n"],
                  help="event_csrmv (headline); coba: the 4000-neuron COBA example; batched: 256 uneven "
                       "networks in persistent cluster launches vs the plain per-network path; jitconn_net: "
                       "4M-neuron just-in-time network; serve: continuous-batching serving loop; sweep: the "
                       "operator sweep (event/sparse csrmv, jitconn) as one JSON line; vmap: a batch of 8 "
                       "spike vectors through one matrix in one launch pair vs 8 sequential calls; stdp: the "
                       "CSR layers' pre/post-spike weight updates; sparse_n: sparse.csrmv transpose=False "
                       "on a dense vector")
  ap.add_argument("--nets", type=int, default=256)
  ap.add_argument("--delay", type=float, default=None,
                  help="coba: synaptic delay (ms) of every projection, as FullProjAlignPostMg(delay=...)")
  ap.add_argument("--sim-steps", type=int, default=0, help="override the workload's number of steps")
  ap.add_argument("--no-forms", action="store_true",
                  help="event_csrmv: skip the batched / served / COBA-example forms reported beside the headline")
  ap.add_argument("--serve-jobs", type=int, default=120, help="jobs of the served stream reported beside the headline")
  return ap.parse_args()


def dist_info():
  ws = int(os.environ.get("WORLD_SIZE", "1"))
  rank = int(os.environ.get("RANK", "0"))
  local = int(os.environ.get("LOCAL_RANK", "0"))
  return ws, rank, local


def load_peaks():
  try:
    with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
      p = json.load(f)
    return float(p["hbm_gbs"]), "measured"
  except Exception:
    return 6800.0, "fallback"


def profile_traffic(name):
  """Per-launch DRAM traffic (bytes) recorded in the committed ncu summary, if any."""
  path = os.path.join(ROOT, "profiles", name)
  try:
    txt = open(path).read()
  except OSError:
    return None
  m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", txt)
  return float(m.group(1)) if m else None


class ClockSampler:
  FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
            "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
            "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

  def __init__(self, gpu_index):
    self.proc = None
    self.gpu = gpu_index
    try:
      self.proc = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.FIELDS}",
                                    "--format=csv,noheader,nounits", "-lms", "100"], stdout=subprocess.PIPE,
                                   stderr=subprocess.DEVNULL, text=True)
    except Exception:
      self.proc = None

  def stop(self):
    if self.proc is None:
      return None
    time.sleep(0.25)
    self.proc.terminate()
    try:
      out, _ = self.proc.communicate(timeout=5)
    except Exception:
      self.proc.kill()
      out, _ = self.proc.communicate()
    rows = [r.split(",") for r in out.strip().splitlines() if r.strip()]
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for r in rows:
      try:
        sm.append(float(r[1]))
        mx = float(r[2])
        for k, nm in enumerate(names):
          if r[5 + k].strip().lower() in ("active", "1"):
            reasons.add(nm)
      except (ValueError, IndexError):
        continue
    if not sm:
      return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(args, device, n_vec=8):
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr, normal_weights
  n, k = args.n, args.fanout
  ind, ptr = fixed_prob_csr(n, n, k, seed=0, device=device)
  if args.weights == "homo":
    data = torch.ones(1, dtype=torch.float32, device=device)
  else:
    data = normal_weights(ind.numel(), 0.5, 0.1, seed=1, device=device)
  spikes = [bernoulli_events(n, args.rate, seed=2 + v, device=device) for v in range(n_vec)]
  return data, ind, ptr, spikes


def same_result(a, b, heter, terms=None):
  """Two results of the same call agree: bit for bit with a homogeneous weight (integer
  counts x w); with per-synapse weights the float32 shared-memory sums are added in a
  run-dependent order, so element by element within 1e-5 of max(|b|, sum of |terms|) (`terms`:
  the same product with |weights|)."""
  if not heter:
    return torch.equal(a, b)
  b = b.to(a.device)
  scale = b.abs() if terms is None else torch.maximum(b.abs(), terms.to(a.device).abs())
  return bool(((a - b).abs() <= 1e-5 * scale.clamp_min(1e-30)).all())


def alg_bytes(n, active, k, heter):
  """Algorithmic bytes of one event.csrmv transpose call on the reference's CSR format:
  spikes (1 B/row) + indptr pair per active row + int32 index per event
  (+ float32 weight per event) + float32 output."""
  e = active * k
  return n + 8 * active + 4 * e + (4 * e if heter else 0) + 4 * n


def headline_config(args, ws=1):
  return {"workload": f"event_csrmv_T N={args.n} K={args.fanout} r={args.rate} {args.weights}",
          "n": args.n, "fanout": args.fanout, "rate": args.rate, "weights": args.weights, "index": "int32",
          "l2": "inputs larger than L2: 8 rotating spike vectors whose segments (8 x ~54 MB) exceed "
                "the 126 MB L2; calls back to back",
          "parallelism": f"replicas x{ws}"}


def run_cpu_baseline(args, data, ind, ptr, spikes, seconds):
  """The reference's CPU path for this operator timed on the host cores: its serial njit
  transpose loop (restated in C), run as independent calls on every host thread at once
  (one spike vector per thread), for about `seconds` of wall time."""
  import oracle
  d = data.cpu().numpy()
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  sp = [s.cpu().numpy() for s in spikes]
  nthr = max(1, oracle.cpu_num_threads())
  batch = np.stack([sp[j % len(sp)] for j in range(nthr)])
  ev_batch = int(sum(int(b.sum()) for b in batch)) * args.fanout
  out = np.zeros((nthr, args.n), np.float32)
  _, used = oracle.cpu_event_csrmv_bool_t_batch(d, ind_h, ptr_h, batch, (args.n, args.n), out)  # warm-up
  t0 = time.perf_counter()
  rounds = 0
  while True:
    oracle.cpu_event_csrmv_bool_t_batch(d, ind_h, ptr_h, batch, (args.n, args.n), out)
    rounds += 1
    if time.perf_counter() - t0 > seconds and rounds >= 2:
      break
  dt = time.perf_counter() - t0
  return {"value": rounds * ev_batch / dt, "unit": UNIT, "cores": int(used), "kind": "port",
          "sample": f"{rounds} rounds of {nthr} concurrent full calls (one per host thread, {used} used) on the "
                    f"same {args.n}x{args.n} CSR, K={args.fanout}, {args.rate:.1%} spike vectors: the reference's "
                    f"serial njit transpose loop (_csr_matvec.py:321-339) restated in C, -O3 -ffast-math, "
                    f"{dt:.1f} s"}


def run_reference(args):
  ws, rank, _ = dist_info()
  if rank != 0:
    return
  import oracle
  oracle.build()
  dev = torch.device("cpu")
  data, ind, ptr, spikes = make_workload(args, dev)
  cpu = run_cpu_baseline(args, data, ind, ptr, spikes, max(3.0, args.cpu_seconds))
  steps, warm = args.steps, args.warmup
  line = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT, "n_gpus": args.gpus,
          "steps": steps, "warmup": warm, "ms_per_step": None, "higher_is_better": True,
          "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
          "config": headline_config(args, args.gpus),
          "cpu_baseline": cpu,
          "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
  mean_events = float(np.mean([int(s.sum()) for s in spikes])) * args.fanout
  line["ms_per_step"] = mean_events / cpu["value"] * 1e3
  print(json.dumps(line))


def main():
  args = parse()
  if args.workload != "event_csrmv":
    fn = {"coba": bench_coba, "batched": bench_batched, "jitconn_net": bench_jitconn_net, "serve": bench_serve,
          "sweep": bench_sweep, "vmap": bench_vmap, "stdp": bench_stdp, "sparse_n": bench_sparse_n}
    line = fn[args.workload](args)
    if line is not None:
      print(json.dumps(line))
    return
  if args.impl == "reference":
    run_reference(args)
    return
  ws, rank, local = dist_info()
  if ws > 1:
    import torch.distributed as dist
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
  device = torch.device("cuda", torch.cuda.current_device())
  from brainpy_gb300 import _lib
  from brainpy_gb300.math import event
  _lib.lib()  # fails loudly when the CUDA library is missing
  n, k = args.n, args.fanout
  data, ind, ptr, spikes = make_workload(args, device)
  active = [int(s.sum()) for s in spikes]
  flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=device)

  def step(i):
    return event.csrmv(data, ind, ptr, spikes[i % len(spikes)], shape=(n, n), transpose=True)

  # Warm-up outside capture builds the plan.  The timed region replays one CUDA graph holding
  # `steps` back-to-back public calls (each the call's two kernels: spike compaction + tiled
  # accumulation) on 8 rotating spike vectors; the segments one rotation touches (8 x ~54 MB)
  # exceed the 126 MB L2, so no call finds its data cached by the previous ones.
  nv = len(spikes)
  side = torch.cuda.Stream(device)
  side.wait_stream(torch.cuda.current_stream(device))
  with torch.cuda.stream(side):
    for i in range(nv):
      step(i)
  torch.cuda.current_stream(device).wait_stream(side)
  torch.cuda.synchronize()

  def capture(idx):
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
      res = [step(i) for i in idx]
    return g, res

  g_warm, _ = capture(range(max(args.warmup, 1)))
  g_run, outs = capture(range(args.steps))
  g_warm.replay()
  torch.cuda.synchronize()
  if ws > 1:
    torch.distributed.barrier()
  clocks = ClockSampler(device.index)
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  torch.cuda.synchronize()
  t_wall = time.perf_counter()
  e0.record()
  g_run.replay()
  e1.record()
  torch.cuda.synchronize()
  t_wall = time.perf_counter() - t_wall
  step_ms = e0.elapsed_time(e1) / args.steps
  # sustained window: the same graph replayed for about a second, each replay timed on its own;
  # the clock sampler runs across both the timed replay and this window
  sus = []
  t_sus = time.perf_counter()
  while time.perf_counter() - t_sus < 1.0 or len(sus) < 20:
    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_.record()
    g_run.replay()
    b_.record()
    sus.append((a_, b_))
    if len(sus) % 50 == 0:
      b_.synchronize()
  torch.cuda.synchronize()
  clk = clocks.stop()
  sus_ms = sorted(a_.elapsed_time(b_) / args.steps for a_, b_ in sus)
  sustained = {"ms_per_step_median": sus_ms[len(sus_ms) // 2], "ms_per_step_min": sus_ms[0],
               "ms_per_step_max": sus_ms[-1], "replays": len(sus_ms), "calls_per_replay": args.steps}
  events_done = sum(active[i % nv] for i in range(args.steps)) * k
  # the graphed results equal eager calls on the same spikes
  heter = args.weights == "heter"
  abs_data = data.abs() if heter else data
  terms = [event.csrmv(abs_data, ind, ptr, spikes[i % nv], shape=(n, n), transpose=True) if heter else None
           for i in range(min(nv, args.steps))]
  for i in range(min(nv, args.steps)):
    assert same_result(outs[i], step(i), heter, terms[i]), "graph replay and eager call disagree"
  # replicas: the slowest rank's time, the events of all ranks
  from brainpy_gb300 import replicas
  step_ms, events_done = replicas.combine(step_ms, events_done)
  value = events_done / (step_ms * 1e-3 * args.steps)

  # The same call alone with L2 flushed before it (one graph per spike vector): the latency
  # of an isolated call, reported beside the sustained figure.
  singles = [capture([i])[0] for i in range(nv)]
  cold = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nv * 2)]
  for j, (a_, b_) in enumerate(cold):
    flush_buf.zero_()
    a_.record()
    singles[j % nv].replay()
    b_.record()
  torch.cuda.synchronize()
  cold_ms = sum(a_.elapsed_time(b_) for a_, b_ in cold) / len(cold)

  # The same `steps` public calls issued eagerly, back to back (no graph: the Python call, the
  # plan-cache lookup and the two launches are in every call), as the median of 20 rounds.
  eager = []
  for _ in range(20):
    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_.record()
    for i in range(args.steps):
      step(i)
    b_.record()
    eager.append((a_, b_))
  torch.cuda.synchronize()
  eager_ms = sorted(a_.elapsed_time(b_) / args.steps for a_, b_ in eager)[len(eager) // 2]

  # e2e through the public API: each step copies its spike vector from pinned host memory,
  # calls event.csrmv on it and copies the result back into pinned host memory.  The steps are
  # captured in one CUDA graph (the copies become graph memcpy nodes), so every byte of every
  # step moves inside the timed region without per-step host dispatch.
  host_spikes = [s.cpu().pin_memory() for s in spikes]
  out_host = [torch.empty(n, dtype=torch.float32).pin_memory() for _ in range(nv)]
  dev_sp = [torch.empty_like(s) for s in spikes]
  w_arg = 1.0 if args.weights == "homo" else data

  def e2e_step(i):
    j = i % nv
    dev_sp[j].copy_(host_spikes[j], non_blocking=True)
    y = event.csrmv(w_arg, ind, ptr, dev_sp[j], shape=(n, n), transpose=True)
    out_host[j].copy_(y, non_blocking=True)

  with torch.cuda.stream(side):
    for i in range(2):
      e2e_step(i)
  torch.cuda.current_stream(device).wait_stream(side)
  torch.cuda.synchronize()
  # Copies on their own streams inside the capture: the upload of step i+1 and the download
  # of step i-1 overlap step i's kernels; a slot's upload waits until the step that last used
  # it has finished its kernels.  Every step's result stays allocated until the replay ends.
  up_s, down_s = torch.cuda.Stream(device), torch.cuda.Stream(device)
  ev_up = [torch.cuda.Event() for _ in range(args.steps)]
  ev_done = [torch.cuda.Event() for _ in range(args.steps)]
  keep = []
  g_e2e = torch.cuda.CUDAGraph()
  with torch.cuda.graph(g_e2e):
    cap = torch.cuda.current_stream(device)
    up_s.wait_stream(cap)
    down_s.wait_stream(cap)
    for i in range(args.steps):
      j = i % nv
      with torch.cuda.stream(up_s):
        if i >= nv:
          up_s.wait_event(ev_done[i - nv])
        dev_sp[j].copy_(host_spikes[j], non_blocking=True)
        ev_up[i].record(up_s)
      cap.wait_event(ev_up[i])
      y = event.csrmv(w_arg, ind, ptr, dev_sp[j], shape=(n, n), transpose=True)
      keep.append(y)
      ev_done[i].record(cap)
      with torch.cuda.stream(down_s):
        down_s.wait_event(ev_done[i])
        out_host[j].copy_(y, non_blocking=True)
    cap.wait_stream(up_s)
    cap.wait_stream(down_s)
  e_start = torch.cuda.Event(enable_timing=True)
  e_end = torch.cuda.Event(enable_timing=True)
  torch.cuda.synchronize()
  e_start.record()
  g_e2e.replay()
  e_end.record()
  e_end.synchronize()
  e2e_ms = e_start.elapsed_time(e_end)
  e2e_events = sum(active[i % nv] for i in range(args.steps)) * k
  torch.cuda.synchronize()
  for j in range(min(nv, args.steps)):  # the results read back are the device results
    assert same_result(out_host[j], outs[j].cpu(), heter, None if terms[j] is None else terms[j].cpu()), \
        "e2e result differs from the device result"
  e2e_ms, e2e_events = replicas.combine(e2e_ms, e2e_events)
  e2e = {"value": e2e_events / (e2e_ms * 1e-3), "unit": UNIT,
         "h2d_bytes_per_step": n + (4 if args.weights == "homo" else 0), "d2h_bytes_per_step": 4 * n}

  peak, peak_kind = load_peaks()
  mean_active = float(np.mean([active[i % len(spikes)] for i in range(args.steps)]))
  kernel_ms = step_ms
  b_alg = alg_bytes(n, mean_active, k, args.weights == "heter")
  achieved = b_alg / (kernel_ms * 1e-3) / 1e9
  roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
          "peak_kind": peak_kind,
          "kernel": ("event_csrmv: compact_blocked_kernel + ecsr_t_split_kernel + split_reduce_kernel (the call's "
                     "three kernels, one bracket)" if launches_per_step(args) == 3 else
                     "event_csrmv: compact_blocked_kernel + ecsr_t_tiled_kernel (the call's two kernels, one bracket)"),
          "timing": "CUDA events around one CUDA-graph replay of all timed calls, back to back",
          "alg_bytes_per_launch": b_alg, "kernel_ms": kernel_ms,
          "traffic": profile_traffic(f"event_csrmv_N1e6_K1000_rate2pct_{args.weights}.md")}
  line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
          "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
          "dtype": "f32", "data": "synthetic",
          "config": headline_config(args, ws),
          "roofline": roof, "e2e": e2e, "gpu_launches": None, "clocks": clk,
          "cold_l2_ms_per_call": cold_ms, "sustained": sustained,
          "eager_ms_per_call": eager_ms,
          "wall_s_timed_loop": t_wall}
  line["gpu_launches"] = args.steps * launches_per_step(args)
  if rank == 0 and ws == 1 and not args.no_cpu_baseline:
    line["cpu_baseline"] = run_cpu_baseline(args, data, ind, ptr, spikes, args.cpu_seconds)
  if rank == 0 and ws == 1 and not args.no_forms:
    del data, ind, ptr, spikes, outs, g_run, g_warm, g_e2e, keep, singles
    event.release_plans()
    torch.cuda.empty_cache()
    line["forms"] = other_forms(args)
  if rank == 0:
    print(json.dumps(line))
  if ws > 1:
    torch.distributed.destroy_process_group()


def other_forms(args):
  """The batched and served forms, the COBA example, the 4M-neuron jitconn network and a 1M-
  neuron CSR network on the whole-GPU runner, each timed with CUDA events under its own clock
  record, summarised beside the headline operator line."""
  import copy
  out = {}
  a = copy.copy(args)
  a.sim_steps = 0
  a.delay = None
  r = bench_coba(a)
  out["coba_example"] = {
      "config": r["config"]["workload"], "runner_steps_per_s": r["value"], "ms_per_step": r["ms_per_step"],
      "per_op_path_steps_per_s": r["per_op_path_steps_per_s"],
      "per_op_graph_steps_per_s": r["per_op_graph_steps_per_s"],
      "cpu_oracle_steps_per_s": r["cpu_baseline"]["value"], "cpu_cores": r["cpu_baseline"]["cores"],
      "runner_vs_per_op": r["value"] / r["per_op_path_steps_per_s"],
      "runner_vs_cpu": r["value"] / r["cpu_baseline"]["value"],
      "firing_rate_hz": r["firing_rate_hz"], "e2e_steps_per_s": r["e2e"]["value"], "clocks": r["clocks"]}
  torch.cuda.empty_cache()
  a = copy.copy(args)
  a.sim_steps = 0
  a.nets = 256
  r = bench_batched(a)
  out["batched_sweep"] = {
      "config": r["config"]["workload"], "network_steps_per_s": r["value"],
      "plain_network_steps_per_s": r["plain_per_network_path"]["value"],
      "plain_sample": r["plain_per_network_path"]["sample"], "speedup_vs_plain": r["speedup_vs_plain"],
      "synaptic_events_per_s": r["synaptic_events_per_s"], "accuracy": r["accuracy"],
      "untuned_network_steps_per_s": r["untuned_form"]["value"], "speedup_vs_untuned": r["speedup_vs_untuned"],
      "tile_choices": r["tuning"]["choices"], "tuning_s": r["tuning"]["seconds"],
      "launches": r["gpu_launches"], "clocks": r["clocks"]}
  torch.cuda.empty_cache()
  a = copy.copy(args)
  a.sim_steps = 200
  r = bench_jitconn_net(a)
  out["jitconn_network"] = {
      "config": r["config"]["workload"] + f", {r['steps']} steps timed", "steps_per_s": r["value"],
      "ms_per_step": r["ms_per_step"], "connections_generated_per_s": r["connections_generated_per_s"],
      "synaptic_events_per_s": r["synaptic_events_per_s"], "firing_rate_hz": r["firing_rate_hz"],
      "push_form": r["push_form"], "stored_form": r["stored_form"], "clocks": r["clocks"]}
  torch.cuda.empty_cache()
  out["large_network"] = bench_large_network()
  torch.cuda.empty_cache()
  from brainpy_gb300 import serve
  a = copy.copy(args)
  a.nets = args.serve_jobs
  clocks = ClockSampler(torch.cuda.current_device())
  r = serve.bench(a)
  clk = clocks.stop()
  out["served_stream"] = {
      "config": r["config"]["workload"], "jobs": r["jobs_done"], "p50_s": r["p50_s"], "p99_s": r["p99_s"],
      "wall_s": r["wall_s"], "network_steps_per_s": r["network_steps_per_s"],
      "synaptic_events_per_s": r["synaptic_events_per_s"],
      "plain_network_steps_per_s": r["plain_per_network_path"]["value"],
      "plain_sample": r["plain_per_network_path"]["sample"], "speedup_vs_plain": r["speedup_vs_plain"],
      "clocks": clk}
  return out


# ---------------------------------------------------------------------------------------
# network workloads
# ---------------------------------------------------------------------------------------
def _cuda_time(fn):
  torch.cuda.synchronize()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record()
  out = fn()
  e1.record()
  e1.synchronize()
  return e0.elapsed_time(e1) * 1e-3, out


def bench_coba(args):
  """The COBA example: 3200 E + 800 I LifRefLTC, 2 % FixedProb, 10000 steps of 0.1 ms."""
  import oracle
  from brainpy_gb300 import dyn
  steps = args.sim_steps or 10000
  V0 = np.random.default_rng(3).normal(-55.0, 5.0, 4000).astype(np.float32)
  net = dyn.EINetwork.fixed_prob(3200, 800, prob=0.02, seed=0, V0=V0)
  tile = int(os.environ.get("BPGPU_NET_TILE", "0")) or None
  dk = dict(delay_e=args.delay, delay_i=args.delay)
  net2 = dyn.EINetwork(net.n, net.n_exc, indices=net.indices, indptr=net.indptr, V0=V0, net_tile=tile, **dk)
  net2.run(100)  # warm-up: plan build, module load
  net2 = dyn.EINetwork(net.n, net.n_exc, indices=net.indices, indptr=net.indptr, V0=V0, net_tile=tile, **dk)
  net2._cluster_plan()  # plan built outside the timed region
  clocks = ClockSampler(torch.cuda.current_device())
  counts = torch.zeros(steps, dtype=torch.int32, device="cuda")
  t_cluster, _ = _cuda_time(lambda: net2.run(steps, spike_counts=counts))
  clk = clocks.stop()
  n_spk = int(counts.sum())
  fan = 64 + 16
  # per-operator path, host loop and CUDA-graph replay, on a bounded number of steps
  k_ops = min(steps, 1000)
  net3 = dyn.EINetwork(net.n, net.n_exc, indices=net.indices, indptr=net.indptr, V0=V0, **dk)
  net3.run(5, method="ops")
  t_ops, _ = _cuda_time(lambda: net3.run(k_ops, method="ops"))
  net4 = dyn.EINetwork(net.n, net.n_exc, indices=net.indices, indptr=net.indptr, V0=V0, **dk)
  net4.run(60, method="ops", graph_steps=50)
  t_graph, _ = _cuda_time(lambda: net4.run(k_ops, method="ops", graph_steps=50))
  # e2e: host V0 in, spike counts out, whole run through the public API
  host_v0 = torch.from_numpy(V0).pin_memory()
  def e2e():
    n5 = dyn.EINetwork(net.n, net.n_exc, indices=net.indices, indptr=net.indptr, V0=host_v0, **dk)
    c, _ = n5.run(steps)
    return c.cpu()
  t_e2e, _ = _cuda_time(e2e)
  # CPU: the oracle's restatement of the reference step, single thread, bounded sample
  st = net.state_numpy()
  st = {k: v.copy() for k, v in net2.state_numpy().items()}
  st["V"][:] = V0
  st["ge"][:] = 0
  st["gi"][:] = 0
  st["t_last"][:] = -1e7
  st["spike"][:] = 0
  ind = net.indices.cpu().numpy()
  ptr = net.indptr.cpu().numpy().astype(np.int64)
  e_end = int(ptr[3200])
  op = oracle.lif_params()
  k_cpu = min(steps, 2000)
  t0 = time.perf_counter()
  csr = (ptr[:3201].astype(np.int32), np.ascontiguousarray(ind[:e_end]), np.float32(0.6),
         (ptr[3200:] - e_end).astype(np.int32), np.ascontiguousarray(ind[e_end:]), np.float32(6.7))
  if args.delay is None:
    oracle.coba_net_run(op, 4000, 3200, *csr, st, 0, k_cpu, np.float32(0.1))
  else:
    oracle.coba_net_run_delayed(op, 4000, 3200, *csr, st, 0, k_cpu, np.float32(0.1), net2.d_e, net2.d_i)
  t_cpu = time.perf_counter() - t0
  return {"metric": "network-steps/s (COBA E/I 4000 neurons, dt 0.1 ms)", "value": steps / t_cluster,
          "unit": "steps/s", "n_gpus": 1, "steps": steps, "warmup": 100, "ms_per_step": t_cluster / steps * 1e3,
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
          "config": {"workload": "COBA 3200E+800I FixedProb(0.02) LifRefLTC, 10000 steps"
                                 + (f", delay {args.delay} ms" if args.delay is not None else ""),
                     "path": "persistent cluster"},
          "synaptic_events_per_s": n_spk * fan / t_cluster, "firing_rate_hz": n_spk / 4000 / (steps * 1e-4),
          "per_op_path_steps_per_s": k_ops / t_ops, "per_op_graph_steps_per_s": k_ops / t_graph,
          "e2e": {"value": steps / t_e2e, "unit": "steps/s", "h2d_bytes_per_step": 4000 * 4 / steps,
                  "d2h_bytes_per_step": 4},
          "cpu_baseline": {"value": k_cpu / t_cpu, "unit": "steps/s", "cores": 1, "kind": "port",
                           "sample": f"{k_cpu} steps of the oracle's float32 restatement (oracle.c orc_coba_net_run)"},
          "clocks": clk, "gpu_launches": 1}


def bench_batched(args):
  """256 independent COBA networks, N ~ logU[1k, 64k], we ~ U[0.3, 1], wi ~ U[3, 10], 5000 steps,
  all in persistent cluster launches, against the plain per-network path (one network at a
  time, one kernel per operator per step, host loop).  The headline form runs autotuned tiles
  (neurons per CTA chosen per size class, tuning outside the timed region) with the launches
  of the different cluster sizes concurrent on side streams; the untuned form (default tiles,
  launches in stream order) is timed from the same initial state beside it."""
  from brainpy_gb300 import dyn
  steps = args.sim_steps or 5000
  rng = np.random.default_rng(11)
  sizes = np.exp(rng.uniform(np.log(1000), np.log(64000), args.nets)).astype(int)
  nets = []
  for k, n in enumerate(sizes):
    ne = int(0.8 * n)
    nets.append(dyn.EINetwork.fixed_prob(ne, n - ne, prob=0.02, we=float(rng.uniform(0.3, 1.0)),
                                         wi=float(rng.uniform(3.0, 10.0)), seed=100 + k,
                                         V0=rng.normal(-55.0, 5.0, n).astype(np.float32),
                                         net_tile=int(os.environ.get("BPGPU_NET_TILE", "0")) or None))
  init = [(x.V.clone(), x.ge.clone(), x.gi.clone(), x.t_last.clone(), x.spike.clone()) for x in nets]
  for x in nets:
    x._cluster_plan()
  k_plain = 20
  # untuned form: the default tile rule, one launch per cluster size in stream order
  counts0 = [torch.zeros(steps, dtype=torch.int32, device="cuda") for _ in nets]
  launches0 = len({x.descriptor().n_tiles for x in nets})
  t_untuned, _ = _cuda_time(lambda: dyn.run_networks(nets, steps, spike_counts=counts0, concurrent=False))
  for x, st in zip(nets, init):
    x.reset_state(*st)
  from brainpy_gb300 import tuning
  t0 = time.perf_counter()
  tune = dyn.autotune_net_tiles(nets, cache=tuning.TuneCache())  # timed afresh (memory-only cache)
  t_tune = time.perf_counter() - t0
  for x in nets:
    x._cluster_plan()
  counts = [torch.zeros(steps, dtype=torch.int32, device="cuda") for _ in nets]
  # the whole run captured as one CUDA graph (the per-size launches as concurrent branches),
  # then launched once; the capture is outside the timed region, writing the descriptors in
  batch = dyn.NetBatch(nets)
  batch.capture(steps)
  clocks = ClockSampler(torch.cuda.current_device())
  t_batch, _ = _cuda_time(lambda: batch.replay(spike_counts=counts))
  clk = clocks.stop()
  same_forms = all(torch.equal(a, b) for a, b in zip(counts0, counts))
  fan = np.array([int(0.8 * n * 0.02) + int((n - int(0.8 * n)) * 0.02) for n in sizes])
  n_spk = np.array([int(c.sum()) for c in counts])
  # plain path: every network from its initial state, k_plain steps each, one after another
  # (warmed up first so that plans and workspaces exist, then reset to the initial state)
  plain = []
  for x, st in zip(nets, init):
    y = dyn.EINetwork(x.n, x.n_exc, indices=x.indices, indptr=x.indptr, we=x.we, wi=x.wi, V0=st[0])
    y.run(1, method="ops")
    y.reset_state(*st)
    plain.append(y)
  pc = []
  def run_plain():
    for y in plain:
      c, _ = y.run(k_plain, method="ops")
      pc.append(c)
  t_plain, _ = _cuda_time(run_plain)
  same = all(torch.equal(c[:k_plain], p) for c, p in zip(counts, pc))
  v_batch = len(nets) * steps / t_batch
  v_plain = len(nets) * k_plain / t_plain
  return {"metric": "network-steps/s (256 uneven COBA networks, batched)", "value": v_batch, "unit": "network-steps/s",
          "n_gpus": 1, "steps": steps, "warmup": 0, "ms_per_step": t_batch / steps * 1e3, "higher_is_better": True,
          "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
          "config": {"workload": f"{len(nets)} networks N~logU[1k,64k], 2% FixedProb, {steps} steps",
                     "neurons_total": int(sizes.sum())},
          "synaptic_events_per_s": float((n_spk * fan).sum()) / t_batch,
          "plain_per_network_path": {"value": v_plain, "unit": "network-steps/s",
                                     "sample": f"all {len(nets)} networks x {k_plain} steps, per-operator kernels, host loop"},
          "speedup_vs_plain": v_batch / v_plain,
          "untuned_form": {"value": len(nets) * steps / t_untuned, "unit": "network-steps/s",
                           "form": "default tiles (a quarter of the network, >= 1024), launches in stream order",
                           "launches": launches0},
          "speedup_vs_untuned": t_untuned / t_batch,
          "tuning": {"seconds": t_tune, "choices": {f"{k:+.1f}": v["choice"] for k, v in tune.items()}},
          "accuracy": ("bit-identical spike counts over the first %d steps of every network: %s; "
                       "tuned+concurrent equals untuned+ordered over all steps: %s") % (k_plain, same, same_forms),
          "form": "tuned tiles; every network's 5000 steps in one CUDA graph launch holding one persistent "
                  "kernel per cluster size as concurrent branches",
          "clocks": clk, "gpu_launches": batch.launches}


def bench_large_network(n=1_000_000, steps=1000):
  """A CSR network larger than one thread-block cluster (1M neurons, 80/20, fan-out 1000, COBA
  weights scaled by 80/1000): the whole-GPU persistent runner (one launch for the run) against
  the per-operator path replayed from CUDA graphs of 50 steps, from the same state; spike
  counts compared step by step."""
  from brainpy_gb300 import dyn
  ne = int(0.8 * n)
  prob = 1000 / n
  V0 = np.random.default_rng(12).normal(-55.0, 5.0, n).astype(np.float32)
  a = dyn.EINetwork.fixed_prob(ne, n - ne, prob=prob, we=0.6 * 0.08, wi=6.7 * 0.08, seed=12, V0=V0)
  b = dyn.EINetwork(a.n, a.n_exc, indices=a.indices, indptr=a.indptr, we=a.we, wi=a.wi, V0=a.V.clone())
  ca = torch.zeros(steps + 50, dtype=torch.int32, device="cuda")
  cb = torch.zeros(steps + 50, dtype=torch.int32, device="cuda")
  a.run(50, method="grid", spike_counts=ca[:50])  # plan, workspace, module load
  b.run(50, method="ops", graph_steps=50, spike_counts=cb[:50])
  clocks = ClockSampler(torch.cuda.current_device())
  t_grid, _ = _cuda_time(lambda: a.run(steps, method="grid", spike_counts=ca[50:]))
  clk = clocks.stop()
  t_ops, _ = _cuda_time(lambda: b.run(steps, method="ops", graph_steps=50, spike_counts=cb[50:]))
  return {"config": f"{n} neurons 80/20, FixedProb fan-out 1000, {steps} steps after 50",
          "grid_runner_steps_per_s": steps / t_grid, "per_op_graph_steps_per_s": steps / t_ops,
          "speedup": t_ops / t_grid, "same_spike_counts": bool(torch.equal(ca, cb)),
          "barrier_waits_ran_out": bool(a.grid_error()),
          "firing_rate_hz": float(ca[50:].double().sum()) / n / (steps * 1e-4), "clocks": clk}


def bench_jitconn_net(args):
  """4M-neuron E/I COBA network (80/20), fan-in 1000 regenerated by event_mv_prob_homo
  (no stored matrix), per-operator path replayed from CUDA graphs of 50 steps."""
  from brainpy_gb300 import dyn
  steps = args.sim_steps or 1000
  n = 4_000_000
  ne = int(0.8 * n)
  p = 1000 / n
  V0 = np.random.default_rng(5).normal(-55.0, 5.0, n).astype(np.float32)
  # COBA's excitatory weight and its inhibitory weight scaled by 80/1000 (the example's 80 inputs
  # a neuron against 1000 here): the network then fires at the ~2 % of neurons a step the
  # workload names (measured at 2.0 % on 200K neurons with this fan-in; COBA's own wi at fan-in
  # 1000, or both weights scaled, silence it after the first volley)
  net = dyn.EINetwork(n, ne, jitconn=dict(prob=p, seeds=(11, 12, 13, 14)), we=0.6, wi=6.7 * 0.08, V0=V0)
  counts = torch.zeros(steps + 60, dtype=torch.int32, device="cuda")
  net.run(60, method="ops", graph_steps=50, spike_counts=counts[:60])
  clocks = ClockSampler(torch.cuda.current_device())
  t, _ = _cuda_time(lambda: net.run(steps, method="ops", graph_steps=50, spike_counts=counts[60:]))
  clk = clocks.stop()
  n_spk = int(counts[60:].sum())
  del net
  torch.cuda.empty_cache()
  # the same network built with the projections' other form (EventJitFPHomoLinear(atomic=True):
  # outdim_parallel=False, an equally distributed realisation of the connectivity), whose
  # step regenerates only the spiking neurons' connections, on the whole-GPU runner
  push = dyn.EINetwork(n, ne, jitconn=dict(prob=p, seeds=(11, 12, 13, 14), outdim_parallel=False), we=0.6,
                       wi=6.7 * 0.08, V0=V0)
  pc = torch.zeros(steps + 60, dtype=torch.int32, device="cuda")
  push.run(60, method="grid", spike_counts=pc[:60])
  t_push, _ = _cuda_time(lambda: push.run(steps, method="grid", spike_counts=pc[60:]))
  p_spk = int(pc[60:].sum())
  push_form = {"steps_per_s": steps / t_push, "ms_per_step": t_push / steps * 1e3,
               "firing_rate_hz": p_spk / n / (steps * 1e-4), "synaptic_events_per_s": p_spk * 1000 / t_push,
               "barrier_waits_ran_out": bool(push.grid_error()),
               "form": "outdim_parallel=False (atomic=True), whole-GPU persistent runner, one launch"}
  del push
  torch.cuda.empty_cache()
  stored_form = bench_jitconn_stored(n, ne, p, V0, steps, counts)
  return {"metric": "network-steps/s (4M-neuron jitconn E/I network)", "value": steps / t, "unit": "steps/s",
          "n_gpus": 1, "steps": steps, "warmup": 60, "ms_per_step": t / steps * 1e3, "higher_is_better": True,
          "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
          "config": {"workload": "4M neurons 80/20, fan-in 1000 via event_mv_prob_homo (outdim_parallel=True), "
                                 "we=0.6 wi=0.536 (COBA's we, its wi x 80/1000: ~2 % firing a step)"},
          "synaptic_events_per_s": n_spk * 1000 / t, "connections_generated_per_s": 4e9 / (t / steps),
          "firing_rate_hz": n_spk / n / (steps * 1e-4), "push_form": push_form, "stored_form": stored_form,
          "clocks": clk}


def bench_jitconn_stored(n, ne, p, V0, steps, counts):
  """The same pull-form network with its connectivity generated once and stored
  (EINetwork.materialize: a presynaptic-row CSR of the same connections), stepped by the
  event-driven CSR products on the per-operator path replayed from CUDA graphs of 50 steps.
  The two products are autotuned (EINetwork.tune_ops) on the spikes after 60 steps; the
  network is then reset and run again from the initial state, and its spike counts are
  compared with the just-in-time run's (`counts`, 60 + `steps` steps).  A failure is
  reported in the form instead of ending the bench."""
  from brainpy_gb300 import dyn
  try:
    jit = dyn.EINetwork(n, ne, jitconn=dict(prob=p, seeds=(11, 12, 13, 14)), we=0.6, wi=6.7 * 0.08, V0=V0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net = jit.materialize()
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    del jit
    mc = torch.zeros(steps + 60, dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    net.run(60, method="ops", graph_steps=50, spike_counts=mc[:60])  # builds the two plans
    torch.cuda.synchronize()
    t_warm = time.perf_counter() - t0
    t0 = time.perf_counter()
    recs = net.tune_ops()
    t_tune = time.perf_counter() - t0
    dev = torch.device("cuda")
    net.reset_state(torch.as_tensor(V0, device=dev), torch.zeros(n, device=dev), torch.zeros(n, device=dev),
                    torch.full((n,), -1e7, device=dev), torch.zeros(n, dtype=torch.bool, device=dev))
    mc.zero_()
    net.run(60, method="ops", graph_steps=50, spike_counts=mc[:60])
    clocks = ClockSampler(torch.cuda.current_device())
    t, _ = _cuda_time(lambda: net.run(steps, method="ops", graph_steps=50, spike_counts=mc[60:]))
    clk = clocks.stop()
    nnz = int(net.indices.numel())
    spk = int(mc[60:].sum())
    out = {"steps_per_s": steps / t, "ms_per_step": t / steps * 1e3, "synapses_stored": nnz,
           "index_bytes": nnz * net.indices.element_size(), "generate_s": t_gen,
           "first_60_steps_s_incl_plan_build": t_warm, "tune_s": t_tune,
           "tuned_choices": {"excitatory_rows": recs[0]["choice"], "inhibitory_rows": recs[1]["choice"]},
           "tuned_times_us": {"excitatory_rows": recs[0]["times_us"], "inhibitory_rows": recs[1]["times_us"]},
           "synaptic_events_per_s_at_mean_out_degree": spk * nnz / n / t,
           "same_spike_counts_as_jitconn": bool(torch.equal(mc, counts)),
           "form": "pull connectivity generated once into a presynaptic-row CSR (bp_jitconn_csr), event-driven "
                   "CSR products, per-operator path from CUDA graphs of 50 steps", "clocks": clk}
    del net
    torch.cuda.empty_cache()
    return out
  except Exception as e:  # noqa: BLE001 -- reported, not raised
    torch.cuda.empty_cache()
    return {"error": f"{type(e).__name__}: {str(e)[:300]}"}


def bench_serve(args):
  from brainpy_gb300 import serve
  return serve.bench(args)


def _graph_time(fn, flush_buf, steps=20):
  """Mean device time of one CUDA-graph replay of fn(), L2 flushed before each replay."""
  side = torch.cuda.Stream()
  side.wait_stream(torch.cuda.current_stream())
  with torch.cuda.stream(side):
    fn()
  torch.cuda.current_stream().wait_stream(side)
  torch.cuda.synchronize()
  g = torch.cuda.CUDAGraph()
  with torch.cuda.graph(g):
    fn()
  for _ in range(3):
    flush_buf.zero_()
    g.replay()
  torch.cuda.synchronize()
  ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
  for a, b in ev:
    flush_buf.zero_()
    a.record()
    g.replay()
    b.record()
  torch.cuda.synchronize()
  return sum(a.elapsed_time(b) for a, b in ev) / steps * 1e-3


def _event_time(fn, flush_buf, steps=20):
  """Mean device time of fn() called eagerly (launch and set-up included), L2 flushed before
  each call."""
  for _ in range(3):
    fn()
  torch.cuda.synchronize()
  ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
  for a, b in ev:
    flush_buf.zero_()
    a.record()
    fn()
    b.record()
  torch.cuda.synchronize()
  return sum(a.elapsed_time(b) for a, b in ev) / steps * 1e-3


def _cusparse_points(ind, ptr, n, k, x, one, flush_buf, peak, ours):
  """torch's CSR SpMV (cuSPARSE) on the same matrix, the homogeneous weight broadcast to every
  entry as the reference's GPU method does (brainpy/_src/math/sparse/_csr_mv.py:197-208):
  y = A x and y = A^T x (A^T as torch's CSC view of A).  Timed eagerly (torch's dispatch and
  cuSPARSE's descriptor set-up are in every call), which matters only at the small sizes.
  Each point carries our sparse.csrmv time on the same product and the largest difference."""
  from brainpy_gb300.math import sparse
  pts = []
  vals = torch.ones(ind.numel(), device="cuda")
  A = torch.sparse_csr_tensor(ptr, ind, vals, (n, n))
  b = 4 * (n + 1) + 8 * ind.numel() + 8 * n
  for T in (False, True):
    M = A.t() if T else A
    try:
      y = torch.mv(M, x)
      t = _event_time(lambda: torch.mv(M, x), flush_buf)
    except (RuntimeError, NotImplementedError) as e:
      pts.append({"op": "cusparse", "T": T, "n": n, "k": k, "unavailable": str(e).splitlines()[0][:160]})
      continue
    ref = sparse.csrmv(one, ind, ptr, x, shape=(n, n), transpose=T)
    diff = float((y - ref).abs().max() / ref.abs().max().clamp_min(1e-30))
    pts.append({"op": "cusparse", "impl": "torch.mv on a CSR tensor" + (" (CSC view)" if T else ""), "T": T,
                "n": n, "k": k, "w": "homo broadcast to nnz", "us": t * 1e6, "nnz_per_s": ind.numel() / t,
                "hbm_frac": b / t / 1e9 / peak, "timing": "eager, CUDA events",
                "ours_us": ours[T] * 1e6, "ours_speedup": t / ours[T], "max_rel_diff": diff})
    del y, ref
  # A^T stored as its own CSR matrix (converted once, outside the timing): cuSPARSE's plain
  # y = B x on B = A^T, the form a user of torch would keep for repeated transposed products
  try:
    B = A.t().to_sparse_csr()
    y = torch.mv(B, x)
    t = _event_time(lambda: torch.mv(B, x), flush_buf)
    ref = sparse.csrmv(one, ind, ptr, x, shape=(n, n), transpose=True)
    diff = float((y - ref).abs().max() / ref.abs().max().clamp_min(1e-30))
    pts.append({"op": "cusparse", "impl": "torch.mv on A^T converted to CSR", "T": True, "n": n, "k": k,
                "w": "homo broadcast to nnz", "us": t * 1e6, "nnz_per_s": ind.numel() / t,
                "hbm_frac": b / t / 1e9 / peak, "timing": "eager, CUDA events", "ours_us": ours[True] * 1e6,
                "ours_speedup": t / ours[True], "max_rel_diff": diff})
    del B, y, ref
  except (RuntimeError, NotImplementedError) as e:
    pts.append({"op": "cusparse", "impl": "A^T converted to CSR", "T": True, "n": n, "k": k,
                "unavailable": str(e).splitlines()[0][:160]})
  del A, vals
  torch.cuda.empty_cache()
  return pts


def bench_sweep(args):
  """The operator sweep: event.csrmv transpose=True on square FixedProb CSR, N in {1e4, 1e5,
  1e6}, K in {100, 1000}, rate in {0.5, 2, 10} %, homogeneous 1.0 / heterogeneous N(0.5, 0.1);
  sparse.csrmv (both orientations) on a dense N(0, 1) vector beside torch's CSR SpMV (cuSPARSE)
  on the same matrix; jitconn event_mv_prob_{homo, uniform, normal} with p = K/N, seed 42, both
  outdim_parallel.  One JSON line with every point."""
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr, normal_weights
  from brainpy_gb300.math import event, jitconn, sparse
  peak, _ = load_peaks()
  flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
  pts = []
  for n in (10_000, 100_000, 1_000_000):
    for k in (100, 1000):
      ind, ptr = fixed_prob_csr(n, n, k, seed=0)
      wh = normal_weights(ind.numel(), 0.5, 0.1, seed=1)
      one = torch.ones(1, device="cuda")
      for rate in (0.005, 0.02, 0.1):
        sp = bernoulli_events(n, rate, seed=2)
        a = int(sp.sum())
        for name, data in (("homo", one), ("heter", wh)):
          t = _graph_time(lambda: event.csrmv(data, ind, ptr, sp, shape=(n, n), transpose=True), flush_buf)
          b = alg_bytes(n, a, k, name == "heter")
          pts.append({"op": "event.csrmv", "T": True, "n": n, "k": k, "rate": rate, "w": name, "us": t * 1e6,
                      "events_per_s": a * k / t, "hbm_frac": b / t / 1e9 / peak})
      x = torch.randn(n, device="cuda")
      b = 4 * (n + 1) + 4 * ind.numel() + 8 * n
      ours = {}
      for T in (True, False):
        ours[T] = _graph_time(lambda: sparse.csrmv(one, ind, ptr, x, shape=(n, n), transpose=T), flush_buf)
        pts.append({"op": "sparse.csrmv", "T": T, "n": n, "k": k, "w": "homo", "us": ours[T] * 1e6,
                    "nnz_per_s": ind.numel() / ours[T], "hbm_frac": b / ours[T] / 1e9 / peak})
      from brainpy_gb300.math.sparse import _csrmv
      for T in (True, False):  # the plain-CSR kernels of the same products (no plan)
        t = _graph_time(lambda: _csrmv(one, ind, ptr, x, (n, n), T, use_plan=False), flush_buf)
        pts.append({"op": "sparse.csrmv", "path": "plain CSR", "T": T, "n": n, "k": k, "w": "homo",
                    "us": t * 1e6, "nnz_per_s": ind.numel() / t, "hbm_frac": b / t / 1e9 / peak})
      pts += _cusparse_points(ind, ptr, n, k, x, one, flush_buf, peak, ours)
      del ind, ptr, wh
      torch.cuda.empty_cache()
      sp = bernoulli_events(n, 0.02, seed=2)
      for fn, kw in ((jitconn.event_mv_prob_homo, dict(weight=1.0)),
                     (jitconn.event_mv_prob_uniform, dict(w_low=0.0, w_high=1.0)),
                     (jitconn.event_mv_prob_normal, dict(w_mu=0.0, w_sigma=1.0))):
        for odp in (True, False):
          t = _graph_time(lambda: fn(sp, conn_prob=k / n, seed=42, shape=(n, n), outdim_parallel=odp, **kw),
                          flush_buf)
          pts.append({"op": fn.__name__, "n": n, "k": k, "rate": 0.02, "outdim_parallel": odp, "us": t * 1e6,
                      "connections_per_s": n * k / t})
  head = [p_ for p_ in pts if p_["op"] == "event.csrmv" and p_["n"] == 1_000_000 and p_["k"] == 1000
          and p_["rate"] == 0.02 and p_["w"] == "homo"][0]
  return {"metric": "operator sweep (event/sparse csrmv transpose, jitconn)", "value": head["events_per_s"],
          "unit": "events/s", "n_gpus": 1, "steps": 20, "warmup": 3, "ms_per_step": head["us"] * 1e-3,
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
          "config": {"workload": "operator sweep; value = event.csrmv T N=1e6 K=1000 r=2% homo",
                     "l2": "flushed before each replay", "timing": "CUDA-graph replay, CUDA events"},
          "points": pts}


def bench_vmap(args, batch=8):
  """A batch of spike vectors through one matrix (the reference maps its primitive over a batch
  with a sequential scan of single calls, brainpy/_src/math/op_register/utils.py:16-38):
  one launch pair for the batch (CSRPlan.csrmv_batch) against `batch` sequential single calls,
  both as CUDA graphs, L2 flushed before each replay."""
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr
  from brainpy_gb300.math import event
  n, k = args.n, args.fanout
  ind, ptr = fixed_prob_csr(n, n, k, seed=0)
  plan = event.prepare(ind, ptr, shape=(n, n))
  w = torch.ones(1, device="cuda")
  ev = torch.stack([bernoulli_events(n, args.rate, seed=2 + b) for b in range(batch)])
  active = int(ev.sum())
  out_b = torch.empty((batch, n), device="cuda")
  out_s = torch.empty((batch, n), device="cuda")

  def batched():
    plan.csrmv_batch(ev, w, out=out_b)

  def sequential():
    for b in range(batch):
      plan.csrmv(ev[b], w, out=out_s[b])

  flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
  t_b = _graph_time(batched, flush_buf, steps=max(args.steps, 20))
  t_s = _graph_time(sequential, flush_buf, steps=max(args.steps, 20))
  torch.cuda.synchronize()
  assert torch.equal(out_b, out_s), "batched rows differ from single calls"
  e = active * k
  return {"metric": "event.csrmv transpose, batch of spike vectors (events/s)", "value": e / t_b, "unit": "events/s",
          "n_gpus": 1, "steps": max(args.steps, 20), "warmup": 3, "ms_per_step": t_b * 1e3, "higher_is_better": True,
          "scaling": "weak", "vs_baseline": None, "dtype": "u32 counts", "data": "synthetic",
          "config": {"workload": f"N={n} K={k} rate={args.rate} homo, batch of {batch} Bernoulli spike vectors",
                     "l2": "flushed before each replay", "timing": "CUDA-graph replay, CUDA events"},
          "sequential_calls": {"value": e / t_s, "ms_per_step": t_s * 1e3},
          "speedup_vs_sequential": t_s / t_b, "gpu_launches": 2}


def bench_stdp(args):
  """STDP weight updates on CSR (brainpy/_src/dnn/linear.py:650-698) at N = 1e6, K = 1000:
  the on-pre update of 2 % spiking rows, in place (what _CSRLayer.stdp_update needs), and the
  functional form that first copies all nnz weights, as the reference's kernel does.
  Algorithmic bytes of the in-place update: the spike vector (1 B/row), an indptr pair per
  spiking row, and per synapse of a spiking row its int32 index, the weight read and written
  and the float32 trace gathered (16 B)."""
  from brainpy_gb300 import dnn
  from brainpy_gb300.connect import bernoulli_events, fixed_prob_csr
  n, k = args.n, args.fanout
  ind, ptr = fixed_prob_csr(n, n, k, seed=0)
  w = torch.full((ind.numel(),), 0.5, device="cuda")
  w2 = torch.empty_like(w)
  sp = bernoulli_events(n, args.rate, seed=2)
  trace = torch.randn(n, device="cuda") * 1e-3
  active = int(sp.sum())
  flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
  t_in = _graph_time(lambda: dnn.csr_on_pre_update(w, ind, ptr, sp, trace, 0.0, 1.0, out=w), flush_buf)
  t_copy = _graph_time(lambda: dnn.csr_on_pre_update(w, ind, ptr, sp, trace, 0.0, 1.0, out=w2), flush_buf)
  peak, _ = load_peaks()
  b = n + 8 * active + 16 * active * k
  return {"metric": "STDP on-pre weight update (synapses updated/s)", "value": active * k / t_in,
          "unit": "synapses/s", "n_gpus": 1, "steps": 20, "warmup": 3, "ms_per_step": t_in * 1e3,
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
          "config": {"workload": f"csr_on_pre_update N={n} K={k} rate={args.rate}, in place",
                     "l2": "flushed before each replay", "timing": "CUDA-graph replay, CUDA events"},
          "roofline": {"bound": "hbm", "achieved": b / t_in / 1e9, "peak": peak, "unit": "GB/s",
                       "frac": b / t_in / 1e9 / peak, "alg_bytes_per_launch": b},
          "functional_copy": {"ms_per_step": t_copy * 1e3, "value": active * k / t_copy,
                              "note": "copies all nnz weights first, as the reference's kernel returns a new array"},
          "gpu_launches": 1}


def bench_sparse_n(args):
  """sparse.csrmv transpose=False, y = A x on a dense vector (brainpy/_src/math/sparse/_csr_mv.py:
  29-108), at --n / --fanout on FixedProb rows: the tiled plan's row-gather kernel plus the
  tile-order reduction.  Algorithmic bytes on the reference's CSR format: indptr, an int32
  index per entry, the vector read and the output written."""
  from brainpy_gb300.connect import fixed_prob_csr
  from brainpy_gb300.math import sparse
  n, k = args.n, args.fanout
  ind, ptr = fixed_prob_csr(n, n, k, seed=0)
  w = torch.ones(1, device="cuda")
  x = torch.randn(n, device="cuda", generator=torch.Generator("cuda").manual_seed(4))
  out = sparse.csrmv(w, ind, ptr, x, shape=(n, n), transpose=False)  # builds and caches the plan
  flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
  t = _graph_time(lambda: sparse.csrmv(w, ind, ptr, x, shape=(n, n), transpose=False), flush_buf)
  peak, _ = load_peaks()
  nnz = ind.numel()
  b = 4 * (n + 1) + 4 * nnz + 4 * n + 4 * n
  return {"metric": "sparse.csrmv transpose=False (matrix entries/s)", "value": nnz / t, "unit": "entries/s",
          "n_gpus": 1, "steps": 20, "warmup": 3, "ms_per_step": t * 1e3, "higher_is_better": True,
          "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
          "config": {"workload": f"sparse_csrmv_N N={n} K={k} homo", "l2": "flushed before each replay",
                     "timing": "CUDA-graph replay, CUDA events", "checksum": float(out.abs().sum())},
          "roofline": {"bound": "hbm", "achieved": b / t / 1e9, "peak": peak, "unit": "GB/s",
                       "frac": b / t / 1e9 / peak, "alg_bytes_per_launch": b},
          "gpu_launches": 2}


def launches_per_step(args):
  """Kernels of ours per event.csrmv transpose call.  A homogeneous weight on >= 2^19 columns
  runs the counting plan: blocked spike compaction, split accumulation (16-bit counters), and
  the reduction of the partial counts; per-synapse weights run the general plan: compaction
  and the cluster-tiled accumulation."""
  from brainpy_gb300.math import event
  return 3 if (args.weights == "homo" and args.n >= event._SPLIT_MIN_N) else 2


if __name__ == "__main__":
  main()
