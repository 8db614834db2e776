"""Independent replicas on several GPUs, one process per GPU.

One scene's exchange does not shard: every order reads all of E_{k-1}, so
splitting the receivers would need an all-gather of E_{k-1} every order.
N GPUs therefore run N independent solves, and a batch of rooms deals its
rooms round-robin to the ranks.  The only communication is on the host
side, over whatever process group torch.distributed was initialised with
(NCCL between GPUs, gloo on CPUs):
* timings reduced to the slowest rank;
* per-room results gathered back in room order.
"""
import os

import torch
import torch.distributed as dist


def env_ranks():
    """(world, rank, local_rank) from the launcher's environment (1, 0, 0 without one)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _active():
    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def shard(items, rank, world):
    """The items rank `rank` of `world` takes: indices rank, rank + world, ...; returns (indices, items)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    idx = list(range(rank, len(items), world))
    return idx, [items[i] for i in idx]


def max_over_ranks(value):
    """The largest value over the ranks (the value itself without a process group)."""
    if value is None or not _active():
        return value
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_in_order(n_items, indices, values):
    """Every rank's (index, value) pairs merged into one list of n_items, in index order, on every rank."""
    pairs = list(zip(indices, values))
    if _active():
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, pairs)
        pairs = [p for part in parts for p in part]
    out = [None] * n_items
    seen = set()
    for i, v in pairs:
        if i in seen or not 0 <= i < n_items:
            raise ValueError(f"item {i} gathered twice or out of range")
        seen.add(i)
        out[i] = v
    if len(seen) != n_items:
        raise ValueError(f"{n_items - len(seen)} items were not produced by any rank")
    return out
