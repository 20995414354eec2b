"""CPU test of the multi-GPU bench logic with two gloo ranks: replicas run
independent chains (distinct seeds) and the job time is the maximum over
ranks; the whole-job value counts every rank's updates."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.reduce_max(1.5 + rank, world)
    seeds = [None] * world
    dist.all_gather_object(seeds, bench.chain_seed(rank))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got, seeds))


def test_two_rank_replicas_reduce_max_and_distinct_seeds():
    torch = pytest.importorskip("torch")
    import multiprocessing as mp
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, seeds in res:
        assert got == 2.5
        assert len(set(seeds)) == 2
    assert torch  # torch.distributed (gloo) is the only collective used
