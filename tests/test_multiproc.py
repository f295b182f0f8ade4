"""Replica path on CPU: two gloo ranks (127.0.0.1) check the batch partition
(complete, disjoint, balanced, identical on every rank) and the job-level
timing reduction that bench.py uses under torchrun."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ddc-svd_gb300"))

from ddcsvd.shard import job_time_ms, problem_cost, shard_batch  # noqa: E402


def _shapes(count=2048, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m = int(rng.integers(16, 257))
        n = int(rng.integers(8, m + 1))
        out.append((m, n))
    return out


def test_shard_single_rank_is_identity():
    s = _shapes(50)
    assert shard_batch(s, 1, 0) == list(range(50))


@pytest.mark.parametrize("world", [2, 3, 4, 8])
def test_shard_partition_balanced(world):
    s = _shapes()
    parts = [shard_batch(s, world, r) for r in range(world)]
    allidx = sorted(i for p in parts for i in p)
    assert allidx == list(range(len(s)))
    loads = [sum(problem_cost(*s[i]) for i in p) for p in parts]
    assert max(loads) / min(loads) <= 1.01


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s = _shapes()
        mine = shard_batch(s, world, rank)
        import torch
        t = torch.zeros(len(s), dtype=torch.int64)
        t[mine] = 1
        dist.all_reduce(t)  # every problem owned exactly once
        local_ms = 10.0 + rank  # rank 1 is the slower one
        job = job_time_ms(local_ms, dist)
        q.put((rank, int(t.min()), int(t.max()), len(mine), job))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    with socket.socket() as sock:
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, tmin, tmax, n, job in res:
        assert tmin == 1 and tmax == 1
        assert job == 11.0
    assert res[0][3] + res[1][3] == 2048
