"""The multi-process path of bench.py (replicas: barrier, max-over-ranks time) on 2 gloo
ranks on the CPU."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip('torch')
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench

    bench.barrier(world)
    out[rank] = bench.max_over_ranks(1.0 + rank, world)
    dist.destroy_process_group()


def test_max_over_ranks_on_two_gloo_ranks():
    port = _free_port()
    ctx = mp.get_context('spawn')
    manager = ctx.Manager()
    out = manager.dict()
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, start_method='spawn', join=True)
    assert dict(out) == {0: 2.0, 1: 2.0}
