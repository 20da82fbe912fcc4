"""Replica bookkeeping of bench.py at world size 2 over gloo (CPU): per-rank seeds,
the job throughput over the slowest rank's time, and the batching form's plasmas
binned over the ranks by particle count."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from pica_gb300.replicas import job_throughput, replica_seed  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    elapsed = [2.0, 5.0][rank]
    value, job = job_throughput(1000, 10, elapsed, dist)
    out.put((rank, replica_seed(7, rank), value, job))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_use_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [7, 8]
    for _, _, value, job in res:
        assert job == 5.0
        assert value == 2 * 1000 * 10 / 5.0


def test_single_rank_without_process_group():
    assert job_throughput(1000, 10, 2.0, None) == (5000.0, 2.0)


def test_bin_members_balances_particles_and_covers_each_plasma_once():
    from pica_gb300.replicas import bin_members
    from pica_gb300 import workloads
    import pica_gb300 as pg
    members = workloads.batched_members(count=64, half=False)
    counts = [sum(pg.plasma_count(s) for s in m["specs"]) for m in members]
    for world in (1, 2, 4, 8):
        bins = bin_members(counts, world)
        flat = sorted(i for b in bins for i in b)
        assert flat == list(range(len(counts)))
        loads = [sum(counts[i] for i in b) for b in bins]
        # largest-first greedy: no rank exceeds the mean by more than the largest plasma
        assert max(loads) <= sum(counts) / world + max(counts)
        assert bins == bin_members(list(counts), world)   # depends only on the counts
    assert bin_members([5, 1, 1, 1, 1, 1], 2) == [[0], [1, 2, 3, 4, 5]]
    assert bin_members([3], 2) == [[0], []]


def _binned_rank(rank, world, port, out):
    from pica_gb300.replicas import bin_members, job_throughput_binned
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    counts = [700, 100, 300, 500, 200, 400]
    mine = bin_members(counts, world)[rank]
    parts = sum(counts[i] for i in mine)
    elapsed = [3.0, 4.0][rank]
    value, job = job_throughput_binned(parts, 10, elapsed, dist)
    out.put((rank, mine, value, job))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_bin_plasmas_and_time_the_job_by_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_binned_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # largest first to the lighter rank: 700 -> r0, 500 -> r1, 400 -> r1 (900), 300 -> r0 (1000),
    # 200 -> r1 (1100), 100 -> r0 (1100)
    assert res[0][1] == [0, 1, 2] and res[1][1] == [3, 4, 5]
    for _, _, value, job in res:
        assert job == 4.0
        assert value == 2200 * 10 / 4.0
