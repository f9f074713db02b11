"""Several GPUs, one process each: the propagation path has no data exchange between
replicas, so ranks work on independent units (networks, jobs, or whole copies of a
workload) and only the measurements are combined."""
import torch
import torch.distributed as dist


def shard(n_units, rank, world):
  """Contiguous range [lo, hi) of n_units that `rank` of `world` processes."""
  if world < 1 or not 0 <= rank < world:
    raise ValueError(f"rank {rank} outside a world of {world}")
  return n_units * rank // world, n_units * (rank + 1) // world


def combine(step_ms, units):
  """(slowest rank's time, units of all ranks): the whole-job figures of a replica run.
  Without an initialised process group (one process) the local values are returned."""
  if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
    return float(step_ms), float(units)
  dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
  t = torch.tensor([float(step_ms)], dtype=torch.float64, device=dev)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
  dist.all_reduce(u)
  return float(t.item()), float(u.item())
