"""Replica sharding and the whole-job reductions, on CPU with gloo ranks."""
import os
import socket

import pytest

from sw2d import replicas


def test_shard_covers_once_and_balances():
    for n in (0, 1, 7, 256, 1000):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(n, r, world) for r in range(world)]
            flat = [i for p in parts for i in p]
            assert flat == list(range(n))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_job_totals_without_group_is_local():
    assert replicas.job_totals(10.0, 2.0) == (10.0, 2.0)
    assert replicas.job_throughput(10.0, 2.0) == 5.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.shard(10, rank, world)
        units = float(sum(100 + i for i in mine))  # a rank's processed units
        seconds = 1.0 + rank                        # the slower rank sets the job time
        q.put((rank, list(mine), replicas.job_totals(units, seconds), replicas.job_throughput(units, seconds)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_sum_units_and_take_max_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    total = float(sum(100 + i for i in range(10)))
    assert res[0][1] + res[1][1] == list(range(10))
    for _, _, (u, s), v in res:
        assert u == total and s == 2.0 and v == total / 2.0
