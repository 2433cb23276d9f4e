"""Host-side logic of the multi-rank paths on CPU (gloo, world size 2).

A single molecule is not sharded (replicas only); batches are: molecules are
split into contiguous ranges of balanced atom counts, each rank builds its
range, and only per-rank counts and timings cross ranks. These tests run the
split and the max-over-ranks timing reduction of bench.py in two gloo
processes.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from sesdf_gb300.partition import split_by_atoms


def test_split_covers_and_balances():
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(500), np.log(50000), 256)).astype(np.int64)
    for ranks in (1, 2, 3, 4, 8):
        parts = split_by_atoms(sizes, ranks)
        assert parts[0][0] == 0 and parts[-1][1] == len(sizes)
        assert all(parts[r][1] == parts[r + 1][0] for r in range(ranks - 1))
        loads = [int(sizes[a:b].sum()) for a, b in parts]
        assert sum(loads) == int(sizes.sum())
        # no rank carries more than its share plus the largest molecule
        assert max(loads) <= sizes.sum() / ranks + sizes.max()


def test_split_edge_cases():
    assert split_by_atoms([], 2) == [(0, 0), (0, 0)]
    assert split_by_atoms([10], 3)[-1][1] == 1
    parts = split_by_atoms([5, 5], 4)
    assert parts[0][0] == 0 and parts[-1][1] == 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, b = split_by_atoms(sizes, world)[rank]
        mine = torch.tensor([a, b, int(np.sum(sizes[a:b]))], dtype=torch.int64)
        got = [torch.zeros(3, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(got, mine)
        # bench.py's timing rule: the slowest rank sets the step time
        t = torch.tensor([1.0 + rank], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        if rank == 0:
            out.put(([g.tolist() for g in got], float(t.item())))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    sizes = np.array([1200, 40, 0, 300, 1, 2500, 6, 700], np.int64)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert parts[0][0] == 0 and parts[1][1] == len(sizes) and parts[0][1] == parts[1][0]
    assert parts[0][2] + parts[1][2] == int(sizes.sum())
    assert tmax == 2.0
