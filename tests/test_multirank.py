"""The multi-rank path of bench.py on CPU with two gloo ranks: every rank
multiplies its own batch (disjoint instances, no collective on the data
path), the step time is the maximum over ranks, and the job's rate counts the
units of all ranks.  The products are checked against Python integers."""
from __future__ import annotations

import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, queue):
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "midint-arithmetic_gb300")):
        sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import oracle
        import workloads

        n, m = 6, 4
        a, b = workloads.mul_pairs(n=n, m=m, seed=bench.rank_seed(workloads.SEED_BASE + 1, rank))
        prod = oracle.mul(a, b, m, True)                       # this rank's batch, no exchange
        ok = np.array_equal(prod, oracle.py_mul(a, b, m, True))
        my_ms = 1.0 + rank                                     # a step time per rank
        bench.barrier(world)
        worst = bench.max_over_ranks(world, my_ms)
        rate = bench.job_rate(world, n, worst)
        queue.put((rank, bool(ok), worst, rate, int(a[0])))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_shard_and_time_like_bench():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(world))
    assert all(ok for _, ok, _, _, _ in res)
    assert all(w == 2.0 for _, _, w, _, _ in res)              # max over ranks
    assert all(abs(r - 2 * 6 / 2e-3) < 1e-6 for _, _, _, r, _ in res)  # all ranks' units / slowest time
    assert res[0][4] != res[1][4]                              # disjoint batches
