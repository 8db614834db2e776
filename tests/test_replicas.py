"""Replica host logic across ranks: two gloo processes on CPU.

The solve does not shard, so several GPUs run independent replicas, and a
batch of rooms is dealt round-robin to the ranks.  These tests check, with
world size 2:
* that every room is taken exactly once;
* that per-room results come back in room order on every rank;
* that timings reduce to the slowest rank.
No GPU is used.
"""
import os
import socket
import tempfile

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from sparrowpy_gb300.batch import shoebox_rooms
    from sparrowpy_gb300.geometry import process_patches, shoebox_room_stub
    from sparrowpy_gb300.replicas import gather_in_order, max_over_ranks, shard
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        rooms = shoebox_rooms(5, seed=3)
        idx, mine = shard(rooms, rank, world)
        # a host-only per-room result: the patch count of the room's geometry
        counts = []
        for room in mine:
            walls = shoebox_room_stub(*room["dims"])
            pts = np.array([w.pts for w in walls])
            nrm = np.array([w.normal for w in walls])
            counts.append(int(process_patches(pts, nrm, room["patch_size"])[0].shape[0]))
        gathered = gather_in_order(len(rooms), idx, counts)
        slowest = max_over_ranks(10.0 + rank)
        np.save(os.path.join(out_dir, f"rank{rank}.npy"),
                np.array([slowest] + [float(c) for c in gathered] + [float(i) for i in idx]))
    finally:
        dist.destroy_process_group()


def test_two_ranks_share_rooms_and_gather_in_order():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from sparrowpy_gb300.batch import shoebox_rooms
    from sparrowpy_gb300.geometry import process_patches, shoebox_room_stub
    rooms = shoebox_rooms(5, seed=3)
    expect = []
    for room in rooms:
        walls = shoebox_room_stub(*room["dims"])
        pts = np.array([w.pts for w in walls])
        nrm = np.array([w.normal for w in walls])
        expect.append(process_patches(pts, nrm, room["patch_size"])[0].shape[0])
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_worker, args=(2, _free_port(), d), nprocs=2, join=True, start_method="spawn")
        r0 = np.load(os.path.join(d, "rank0.npy"))
        r1 = np.load(os.path.join(d, "rank1.npy"))
    assert r0[0] == r1[0] == 11.0                       # the slowest rank's time on both
    np.testing.assert_array_equal(r0[1:6], expect)       # every room, in order, on rank 0
    np.testing.assert_array_equal(r1[1:6], expect)       # and on rank 1
    np.testing.assert_array_equal(r0[6:], [0, 2, 4])     # rank 0 took rooms 0, 2, 4
    np.testing.assert_array_equal(r1[6:], [1, 3])        # rank 1 took rooms 1, 3


def test_shard_and_gather_single_process():
    from sparrowpy_gb300.replicas import gather_in_order, max_over_ranks, shard
    items = list("abcdefg")
    parts = [shard(items, r, 3) for r in range(3)]
    assert sorted(i for idx, _ in parts for i in idx) == list(range(7))
    assert parts[1] == ([1, 4], ["b", "e"])
    assert gather_in_order(3, [2, 0, 1], ["z", "x", "y"]) == ["x", "y", "z"]
    with pytest.raises(ValueError):
        gather_in_order(3, [0, 1], ["x", "y"])         # a missing item
    with pytest.raises(ValueError):
        shard(items, 3, 3)
    assert max_over_ranks(2.5) == 2.5 and max_over_ranks(None) is None
