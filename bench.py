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


def alg_bytes(n, active, k, heter):
  """Algorithmic bytes of one event.csrmv transpose call on the reference's CSR format:
  spikes (1 B/row) + indptr pair per active row + int32 index per event
  (+ float32 weight per event) + float32 output."""
  e = active * k
  return n + 8 * active + 4 * e + (4 * e if heter else 0) + 4 * n


def run_cpu_baseline(args, data, ind, ptr, spikes, seconds):
  import oracle
  d = data.cpu().numpy()
  ind_h, ptr_h = ind.cpu().numpy(), ptr.cpu().numpy()
  sp = [s.cpu().numpy() for s in spikes]
  out = np.zeros(args.n, np.float32)
  oracle.cpu_event_csrmv_bool(d, ind_h, ptr_h, sp[0], (args.n, args.n), True, out)  # warm-up
  t0 = time.perf_counter()
  calls, events = 0, 0
  while True:
    s = sp[calls % len(sp)]
    oracle.cpu_event_csrmv_bool(d, ind_h, ptr_h, s, (args.n, args.n), True, out)
    calls += 1
    events += int(s.sum()) * args.fanout
    if time.perf_counter() - t0 > seconds and calls >= 3:
      break
  dt = time.perf_counter() - t0
  return {"value": events / dt, "unit": UNIT, "cores": 1, "kind": "port",
          "sample": f"{calls} full calls on the same {args.n}x{args.n} CSR, K={args.fanout}, "
                    f"{args.rate:.1%} spike vectors: the reference's serial njit transpose loop "
                    f"(_csr_matvec.py:321-339) restated in C, -O3 -ffast-math, {dt:.1f} s"}


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
          "config": {"workload": f"event_csrmv_T N={args.n} K={args.fanout} r={args.rate} {args.weights}"},
          "cpu_baseline": cpu,
          "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
  mean_events = float(np.mean([int(s.sum()) for s in spikes])) * args.fanout
  line["ms_per_step"] = mean_events / cpu["value"] * 1e3
  print(json.dumps(line))


def main():
  args = parse()
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
  L = _lib.lib()
  n, k = args.n, args.fanout
  data, ind, ptr, spikes = make_workload(args, device)
  active = [int(s.sum()) for s in spikes]
  flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=device)
  out = torch.empty(n, dtype=torch.float32, device=device)

  def step(i):
    return event._event_csrmv(data, ind, ptr, spikes[i % len(spikes)], (n, n), True, _lib.BP_EV_F32_POS, out=out)

  for i in range(args.warmup):
    step(i)
  torch.cuda.synchronize()
  starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
  ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
  if ws > 1:
    torch.distributed.barrier()
  clocks = ClockSampler(device.index)
  torch.cuda.synchronize()
  L.bp_timer_enable(1)
  t_wall = time.perf_counter()
  events_done = 0
  for i in range(args.steps):
    flush_buf.zero_()
    starts[i].record()
    step(i)
    ends[i].record()
    events_done += active[i % len(spikes)] * k
  torch.cuda.synchronize()
  t_wall = time.perf_counter() - t_wall
  import ctypes
  kt_ms, kt_n = ctypes.c_double(), ctypes.c_int64()
  _lib.check(L.bp_timer_collect(ctypes.byref(kt_ms), ctypes.byref(kt_n)), "timer")
  L.bp_timer_enable(0)
  clk = clocks.stop()
  step_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
  if ws > 1:
    t = torch.tensor([step_ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    step_ms = float(t)
    ev_t = torch.tensor([events_done], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(ev_t)
    events_done = float(ev_t)
  value = events_done / (step_ms * 1e-3)

  # e2e through the public API: host spike vector (pinned) -> device, result -> host
  host_spikes = [s.cpu().pin_memory() for s in spikes]
  out_host = torch.empty(n, dtype=torch.float32).pin_memory()
  for i in range(2):
    y = event.csrmv(1.0 if args.weights == "homo" else data, ind, ptr, host_spikes[i], shape=(n, n), transpose=True)
    out_host.copy_(y)
  torch.cuda.synchronize()
  e_start = torch.cuda.Event(enable_timing=True)
  e_end = torch.cuda.Event(enable_timing=True)
  e2e_events = 0
  e2e_ms = 0.0
  for i in range(args.steps):
    flush_buf.zero_()
    e_start.record()
    y = event.csrmv(1.0 if args.weights == "homo" else data, ind, ptr, host_spikes[i % len(spikes)], shape=(n, n),
                    transpose=True)
    out_host.copy_(y, non_blocking=True)
    e_end.record()
    e_end.synchronize()
    e2e_ms += e_start.elapsed_time(e_end)
    e2e_events += active[i % len(spikes)] * k
  e2e = {"value": e2e_events / (e2e_ms * 1e-3), "unit": UNIT,
         "h2d_bytes_per_step": n + (4 if args.weights == "homo" else 0), "d2h_bytes_per_step": 4 * n}

  peak, peak_kind = load_peaks()
  mean_active = float(np.mean([active[i % len(spikes)] for i in range(args.steps)]))
  kernel_ms = kt_ms.value / max(kt_n.value, 1)
  b_alg = alg_bytes(n, mean_active, k, args.weights == "heter")
  achieved = b_alg / (kernel_ms * 1e-3) / 1e9
  roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
          "peak_kind": peak_kind,
          "kernel": "event_csrmv: compact_blocked_kernel + ecsr_t_tiled_kernel (the call's two kernels, one bracket)",
          "alg_bytes_per_launch": b_alg, "kernel_ms": kernel_ms,
          "traffic": profile_traffic(f"event_csrmv_N1e6_K1000_r2_{args.weights}.md")}
  line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
          "ms_per_step": step_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
          "dtype": "f32", "data": "synthetic",
          "config": {"workload": f"event_csrmv_T N={n} K={k} r={args.rate} {args.weights}",
                     "n": n, "fanout": k, "rate": args.rate, "weights": args.weights, "index": "int32",
                     "l2": "flushed between timed steps (256 MB write); 8 rotating spike vectors",
                     "parallelism": f"replicas x{ws}"},
          "roofline": roof, "e2e": e2e, "gpu_launches": None, "clocks": clk,
          "wall_s_timed_loop": t_wall}
  line["gpu_launches"] = args.steps * launches_per_step(args)
  if rank == 0 and ws == 1 and not args.no_cpu_baseline:
    line["cpu_baseline"] = run_cpu_baseline(args, data, ind, ptr, spikes, args.cpu_seconds)
  if rank == 0:
    print(json.dumps(line))
  if ws > 1:
    torch.distributed.destroy_process_group()


def launches_per_step(args):
  """Kernels of ours per event.csrmv transpose call on the tiled plan (the path the
  front-end takes for this size): blocked spike compaction + tiled accumulation."""
  return 2


if __name__ == "__main__":
  main()
