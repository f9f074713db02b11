"""Replica runs on several processes (gloo on CPU, world size 2): the work split and the
combination of the ranks' measurements used by bench.py under torchrun."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
  with socket.socket() as s:
    s.bind(("127.0.0.1", 0))
    return s.getsockname()[1]


def _rank(rank, world, port, q):
  import torch.distributed as dist
  from brainpy_gb300 import replicas
  os.environ["MASTER_ADDR"] = "127.0.0.1"
  os.environ["MASTER_PORT"] = str(port)
  dist.init_process_group("gloo", rank=rank, world_size=world)
  try:
    lo, hi = replicas.shard(10, rank, world)
    t, u = replicas.combine(step_ms=1.5 + rank, units=hi - lo)
    q.put((rank, lo, hi, t, u))
  finally:
    dist.destroy_process_group()


def test_two_replicas_gloo():
  ctx = mp.get_context("spawn")
  q = ctx.Queue()
  port = _free_port()
  procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
  for p in procs:
    p.start()
  res = sorted(q.get(timeout=120) for _ in procs)
  for p in procs:
    p.join(timeout=60)
    assert p.exitcode == 0
  assert [(r[1], r[2]) for r in res] == [(0, 5), (5, 10)]
  for r in res:
    assert r[3] == 2.5 and r[4] == 10.0  # slowest rank's time, units of both ranks


def test_single_process():
  from brainpy_gb300 import replicas
  assert replicas.combine(3.0, 7) == (3.0, 7.0)
  assert replicas.shard(7, 0, 1) == (0, 7)
  with pytest.raises(ValueError):
    replicas.shard(7, 2, 2)
