"""The benchmark's multi-rank host logic on CPU (gloo, world size 2): one
process per GPU runs an independent replica, the timed region is bracketed
by barriers, and the slowest rank's time is the one reported.  The replicas
exchange nothing else -- a single scene does not shard -- so these helpers
are the whole N > 1 path."""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    assert bench.dist_info() == (rank, world, rank)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench._barrier(world)
    got = bench._max_over_ranks(1.5 + rank, world, torch.device("cpu"))
    bench._barrier(world)
    out.put((rank, got))
    dist.destroy_process_group()


def test_slowest_rank_is_reported_on_every_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = dict(q.get(timeout=5) for _ in procs)
    assert got == {0: 2.5, 1: 2.5}


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    bench._barrier(1)
    assert bench._max_over_ranks(3.25, 1, None) == 3.25
