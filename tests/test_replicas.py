"""The multi-GPU path is replicas only (one cavity per GPU, no exchange): the
bench's barrier and max-over-ranks timing, checked with two gloo ranks on CPU."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    import sys
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
    q.put((rank, ms, bench.replica_value(ms, world)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_max_over_ranks_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[1] for g in got] == [15.0, 15.0]   # every rank sees the slowest rank's time
    assert [g[2] for g in got] == [7.5, 7.5]     # two replicas: half the time per cavity-step


def test_single_rank_is_identity():
    import sys
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
    assert bench.replica_value(12.5, 1) == 12.5


def _batch_rank(rank: int, world: int, port: int, q):
    import sys
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "cfd-bench_gb300"))
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cases = bench.batch_cases(96)
    mine = bench.shard_cases(len(cases), rank, world)
    cells = sum(cases[i]["imax"] * cases[i]["jmax"] * cases[i]["kmax"] for i in mine)
    ids = [None] * world
    dist.all_gather_object(ids, mine)
    # each rank's share is stepped for 10 steps in a wall time that differs per rank
    updates, wall = bench.batch_totals(float(cells * 10), 1.0 + rank, world, "cpu")
    q.put((rank, ids, cells, updates, wall))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_batch_instances_shard_across_two_gloo_ranks():
    """The batch workload under N ranks: every instance is stepped by exactly
    one rank (ids rank, rank + N, ...), with no exchange between ranks; the
    aggregate rate is all ranks' cell updates over the slowest rank's time."""
    import sys
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "cfd-bench_gb300"))
    import bench
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_batch_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    ids = got[0][1]
    assert ids == got[1][1]  # both ranks see the same partition
    assert sorted(ids[0] + ids[1]) == list(range(96)) and not set(ids[0]) & set(ids[1])
    cases = bench.batch_cases(96)
    total = sum(c["imax"] * c["jmax"] * c["kmax"] for c in cases)
    assert got[0][2] + got[1][2] == total
    for _, _, _, updates, wall in got:
        assert updates == float(total * 10)
        assert wall == 2.0  # the slowest rank's time
    assert bench.shard_cases(5, 0, 1) == [0, 1, 2, 3, 4]
