"""CPU: sharding a batch of uneven beams across ranks (one GPU each).

Beams are independent, so a multi-GPU batch is each rank running its own
shard with no data-path collective.  Two gloo ranks on CPU check that every
rank derives the same partition on its own, that the shards are disjoint and
cover the batch, that the points are balanced, that each rank's shard plan
(the library's own work-queue planner, lp_batch_plan, which makes no CUDA
call) covers exactly its beams' tiles and points, and that gathering the
per-rank results (oracle propagation of each shard's beams) reproduces the
single-rank run.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from lightprop2d_gb300.batch import partition_beams, plan_info, shard
from oracle import lp_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _beam(i, n):
    f0 = O.random_phase_hole(n, 500 * O.um, 150 * O.um, seed=100 + i)
    g = O.grids(500 * O.um, n, 632 * O.nm)
    _, x = O.propagate(O.fft2(f0), g["Kz"], 0.5 + 0.1 * i)
    return float(np.sum(np.abs(x) ** 2)), complex(x[n // 2, n // 3])


SIZES = [64, 16, 32, 64, 16, 16, 32, 64, 16, 32, 16, 64, 32]
# the uneven batch's size mix (64% 256^2, 25% 512^2, 9% 1024^2, 2% 2048^2), 100 beams
BATCH = [256] * 64 + [512] * 25 + [1024] * 9 + [2048] * 2
TILE_POINTS = 4096  # points per batch tile (lp_batch.cu)


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        parts = partition_beams(SIZES, world)
        mine = {i: _beam(i, SIZES[i]) for i in parts[rank]}
        # this rank's shard of the uneven batch, planned by the library
        own = shard(BATCH, world, rank)
        sizes = [BATCH[i] for i in own]
        plan = plan_info(sizes, 0.1, 632e-7, [0.5 + 0.01 * i for i in own],
                         lens_f=[5.0] * len(own))
        gathered = [None] * world
        dist.all_gather_object(gathered, (parts, mine, own, plan))
        if rank == 0:
            q.put(gathered)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_partition_is_complete_disjoint_balanced():
    for world in (1, 2, 3, 4, 8):
        sizes = [256] * 7 + [2048] * 3 + [512] * 11 + [1024] * 5
        parts = partition_beams(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] ** 2 for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes) ** 2
        assert parts == partition_beams(sizes, world)
    with pytest.raises(ValueError):
        partition_beams([256], 0)
    assert partition_beams([], 2) == [[], []]


def test_two_gloo_ranks_reproduce_single_rank():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    parts = [g[0] for g in gathered]
    assert parts[0] == parts[1]
    # shard plans: disjoint, covering, each exactly its beams' 3 passes of tiles
    owns = [set(g[2]) for g in gathered]
    assert not (owns[0] & owns[1]) and sorted(owns[0] | owns[1]) == list(range(len(BATCH)))
    total = plan_info(BATCH, 0.1, 632e-7, 1.0)
    for own, plan in ((g[2], g[3]) for g in gathered):
        pts = sum(BATCH[i] ** 2 for i in own)
        assert plan["points"] == pts
        assert plan["tiles"] == 3 * pts // TILE_POINTS
        assert plan["items"] > 0
    assert sum(g[3]["points"] for g in gathered) == total["points"]
    assert sum(g[3]["tiles"] for g in gathered) == total["tiles"]
    loads = [g[3]["points"] for g in gathered]
    assert max(loads) - min(loads) <= max(BATCH) ** 2
    merged = {}
    for _, mine, _, _ in gathered:
        assert not (set(mine) & set(merged))
        merged.update(mine)
    assert sorted(merged) == list(range(len(SIZES)))
    for i, n in enumerate(SIZES):
        e, v = _beam(i, n)
        assert merged[i][0] == pytest.approx(e, rel=1e-12)
        assert merged[i][1] == v
