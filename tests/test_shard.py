"""The batched forms' multi-GPU plan on CPU: whole tiles dealt to ranks by size (every rank
computes the same plan), and the max-over-ranks timing, on world_size-2 gloo process groups."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from game_engine_gb300 import shard, workloads


def test_plan_partitions_and_balances():
    sides = workloads.tile_sides(4096, workloads.SEEDS["tiles_4096"])
    cells = [s * s for s in sides]
    for world in (1, 2, 3, 8):
        shards = shard.plan(cells, world)
        flat = sorted(k for s in shards for k in s)
        assert flat == list(range(len(cells)))
        loads = shard.loads(cells, shards)
        # LPT's bound: the heaviest rank within 4/3 of the mean (and of the largest tile)
        assert max(loads) <= max(4 / 3 * sum(cells) / world, max(cells)) + max(cells)
        assert max(loads) - min(loads) <= max(cells)


def test_plan_edge_cases():
    assert shard.plan([], 2) == [[], []]
    assert shard.plan([5], 3) == [[0], [], []]
    assert shard.plan([4, 4, 4, 4], 2) == [[0, 2], [1, 3]]  # ties to the lower rank
    with pytest.raises(ValueError):
        shard.plan([1], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sides = workloads.tile_sides(256, workloads.SEEDS["tiles_256_adjoint"],
                                     workloads.ADJOINT_TILE_SIDES)
        cells = [s * s for s in sides]
        mine = shard.plan(cells, world)[rank]
        plans = [None] * world
        dist.all_gather_object(plans, mine)
        slowest = shard.max_over_ranks(10.0 + rank)
        q.put((rank, plans, slowest, sum(cells[k] for k in mine)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_agree_on_the_plan_and_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    plans = [g[1] for g in got]
    assert plans[0] == plans[1]  # both ranks see both shards the same
    a, b = plans[0]
    assert not set(a) & set(b) and len(a) + len(b) == 256
    assert all(g[2] == 11.0 for g in got)  # the max over ranks reaches both
    assert abs(got[0][3] - got[1][3]) <= 512 * 512
