"""Replica bookkeeping of bench.py at world size 2 over gloo (CPU): per-rank seeds
and the job throughput over the slowest rank's time."""
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
