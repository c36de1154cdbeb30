"""Scene sharding for one process per GPU (host logic, on CPU).

The multi-GPU form of the sweep partitions independent scenes across ranks
with no data-path collective; these tests cover the partition and its use by
two gloo ranks (world size 2) that each take their share and agree on the
total through host-side collectives only.
"""
from __future__ import annotations

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from sphnj_gb300 import cases
from sphnj_gb300.sharding import balanced_partition, loads


def sweep_weights():
    out = []
    for s in range(cases.SWEEP_SCENES):
        p = cases.sweep_scene(s).params()
        out.append(p.fluid_number_total + p.solid_number)
    return out


def test_partition_covers_every_scene_once():
    w = [5, 3, 9, 1, 1, 7, 2, 8]
    for n in (1, 2, 3, 8, 11):
        parts = balanced_partition(w, n)
        assert len(parts) == n
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(w)))


def test_partition_balance_bound_on_the_sweep():
    w = sweep_weights()
    for n in (2, 4, 8):
        parts = balanced_partition(w, n)
        ld = loads(w, parts)
        assert max(ld) <= sum(w) / n + max(w)
        assert max(ld) / (sum(w) / n) < 1.05  # 256 scenes: within 5% of perfect balance


def test_partition_is_deterministic():
    w = sweep_weights()
    assert balanced_partition(w, 4) == balanced_partition(list(w), 4)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, weights, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = balanced_partition(weights, world)[rank]
        local = torch.tensor([sum(weights[i] for i in mine), len(mine)], dtype=torch.int64)
        total = local.clone()
        dist.all_reduce(total, op=dist.ReduceOp.SUM)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        slowest = torch.tensor([float(local[0])])  # stands in for a rank's timed region
        dist.all_reduce(slowest, op=dist.ReduceOp.MAX)
        out_q.put((rank, int(total[0]), int(total[1]), gathered, float(slowest[0])))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_the_sweep():
    weights = sweep_weights()
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, weights, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total_w, total_n, gathered, slowest in res:
        assert total_w == sum(weights)
        assert total_n == len(weights)
        flat = sorted(i for part in gathered for i in part)
        assert flat == list(range(len(weights)))
        assert slowest == max(loads(weights, balanced_partition(weights, world)))
