"""bench.py's replica plumbing on CPU: two gloo ranks, per-rank device mapping, max over ranks."""
from __future__ import annotations

import os
import socket

import pytest

from conftest import ROOT


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, str(ROOT))
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="3,5")
    import bench
    r, w, D = bench._replica_setup(cuda=False)
    m = bench._max_over_ranks(D, float(10 + rank))
    q.put((r, w, os.environ["CUDA_VISIBLE_DEVICES"], m))
    D.barrier()
    D.destroy_process_group()


def test_two_replicas_map_devices_and_reduce_max():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, "3", 11.0), (1, 2, "5", 11.0)]


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, str(ROOT))
    import bench
    env = {k: os.environ.pop(k) for k in ("RANK", "WORLD_SIZE") if k in os.environ}
    try:
        assert bench._replica_setup(cuda=False) == (0, 1, None)
        assert bench._max_over_ranks(None, 3.5) == 3.5
    finally:
        os.environ.update(env)
