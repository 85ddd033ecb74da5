"""How the batched forms spread over several GPUs: whole tiles to ranks, no exchange.

Tiles are independent (each steps exactly as a DeviceStep of its size would), so a multi-GPU
batched run deals whole tiles to the ranks and never communicates while it ticks: a size-balanced
greedy (largest tiles first, each to the rank with the fewest cells so far; Graham's LPT rule, within
4/3 of the best balance) decides which rank holds which tile, every rank computes the same plan
from the same sizes, and the host gathers the per-tile hashes or gradients at the end. One large
tile does not shard here: on one GPU a run of it is a replica.
"""
from __future__ import annotations

import heapq


def plan(cells, world: int):
    """Tile indices a rank, each list in index order, for tiles of `cells` cells over `world`
    ranks. Ties go to the lower rank, so every rank computes the same plan."""
    if world < 1:
        raise ValueError("world must be at least 1")
    order = sorted(range(len(cells)), key=lambda k: (-int(cells[k]), k))
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        out[r].append(k)
        heapq.heappush(heap, (load + int(cells[k]), r))
    return [sorted(s) for s in out]


def loads(cells, shards):
    return [sum(int(cells[k]) for k in s) for s in shards]


def max_over_ranks(value: float) -> float:
    """The largest of every rank's value (a timing's max over ranks), or the value alone when no
    process group is up."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
