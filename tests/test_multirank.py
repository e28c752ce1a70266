"""The multi-rank path of bench.py on CPU with two gloo ranks.

Every rank multiplies its own contiguous range of the job's instances
(disjoint, no collective on the data path) and its own part of the job's
ragged list (split by estimated work); the step time is the maximum over
ranks and the job's rate counts the units of all ranks.  The oracle stands in
for the GPU kernels; the products gathered from both ranks are checked
against the oracle run over the whole job.  The launcher decision of
`--gpus N` and the torchrun command it starts are checked too."""
from __future__ import annotations

import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _ragged_results(oracle, ops, pool):
    """Each op's result limbs (and carry-out for additions) by the oracle."""
    res = []
    for op in ops:
        la, lb = int(op["la"]), int(op["lb"])
        x = pool[int(op["a_off"]):int(op["a_off"]) + la]
        y = pool[int(op["b_off"]):int(op["b_off"]) + lb]
        m = max(la, lb)
        xp, yp = np.pad(x, (0, m - la)), np.pad(y, (0, m - lb))
        if op["kind"] == 0:
            r, c = oracle.add(xp, yp, m)
            res.append((r.tobytes(), int(c[0])))
        else:
            res.append((oracle.mul(xp, yp, m, full=True)[: la + lb].tobytes(), 0))
    return res


def _rank_main(rank, world, port, queue):
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "midint-arithmetic_gb300")):
        sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import oracle
        import workloads

        # plain batches: this rank's instance range of the job's batch
        n, m = 6, 4
        lo, hi = bench.instance_range(n, rank)
        a, b = workloads.mul_pairs(n=n, m=m, first=lo)
        prod = oracle.mul(a, b, m, True)                       # this rank's batch, no exchange
        my_ms = 1.0 + rank                                     # a step time per rank
        bench.barrier(world)
        worst = bench.max_over_ranks(world, my_ms)
        rate = bench.job_rate(world, n, worst)

        # ragged: this rank's part of the job's list, its ops' global indices and results
        ops, pool, _ = bench.ragged_shard(20, world, rank)
        res = _ragged_results(oracle, ops, pool)
        gathered = [None] * world
        dist.all_gather_object(gathered, {"range": (lo, hi), "prod": prod.tobytes(),
                                          "ragged": [(int(o["kind"]), int(o["la"]), int(o["lb"])) for o in ops],
                                          "n_ops": ops.size})
        queue.put((rank, worst, rate, gathered, len(res)))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(180)
def test_two_gloo_ranks_shard_and_time_like_bench():
    import bench
    import oracle
    import workloads

    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=150) for _ in range(world)), key=lambda r: r[0])
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert all(w == 2.0 for _, w, _, _, _ in res)              # max over ranks
    assert all(abs(r - 2 * 6 / 2e-3) < 1e-6 for _, _, r, _, _ in res)  # all ranks' units / slowest time
    g = res[0][3]
    assert g == res[1][3]                                      # both ranks gathered the same
    # disjoint contiguous instance ranges covering the job; products equal the oracle over the job
    assert [x["range"] for x in g] == [(0, 6), (6, 12)]
    a, b = workloads.mul_pairs(n=12, m=4)
    want = oracle.mul(a, b, 4, True)
    got = np.frombuffer(b"".join(x["prod"] for x in g), np.uint64)
    assert np.array_equal(got, want)
    assert np.array_equal(want, oracle.py_mul(a, b, 4, True))
    # the ragged list of the job (2 x 20 ops) split once, every op on exactly one rank
    assert sum(x["n_ops"] for x in g) == 40
    full_ops, _, _ = workloads.ragged_ops(n_ops=40)
    job = sorted((int(o["kind"]), int(o["la"]), int(o["lb"])) for o in full_ops)
    assert sorted(t for x in g for t in x["ragged"]) == job


def test_ragged_split_is_balanced_and_exact():
    import bench
    import workloads

    ops, _, _ = workloads.ragged_ops(n_ops=200000)
    work = bench.ragged_work_estimate(ops["kind"], ops["la"], ops["lb"])
    for world in (2, 4, 8):
        parts = bench.shard_ragged(work, world)
        idx = np.concatenate(parts)
        assert idx.size == ops.size and np.unique(idx).size == ops.size
        loads = np.array([work[p].sum() for p in parts])
        assert loads.max() / loads.mean() < 1.01, loads        # within 1 % of the mean
        assert all(np.all(np.diff(p) > 0) for p in parts)      # list order kept
    # one rank: the list is exactly the workload generator's
    ops1, pool1, out1 = bench.ragged_shard(5000, 1, 0)
    ops0, pool0, out0 = workloads.ragged_ops(n_ops=5000)
    assert np.array_equal(ops1, ops0) and np.array_equal(pool1, pool0) and out1 == out0


def test_work_estimate_orders_sizes():
    import bench

    k = np.array([0, 0, 1, 1, 1], np.uint32)
    la = np.array([4, 1024, 4, 128, 1024], np.uint32)
    lb = np.array([4, 1024, 4, 128, 1024], np.uint32)
    w = bench.ragged_work_estimate(k, la, lb)
    assert w[0] < w[1] and w[2] < w[3] < w[4]
    assert w[1] < w[4]                                          # a 1024-limb add is cheaper than the product


def test_gpus_flag_launches_or_refuses(monkeypatch):
    import bench

    monkeypatch.delenv("WORLD_SIZE", raising=False)
    assert bench.check_world(1, 1) is None
    assert bench.check_world(4, 1) == "launch"                  # no launcher: re-exec under torchrun
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.check_world(2, 2) is None
    assert "launcher started 2" in bench.check_world(4, 2)      # a launcher with another count: refuse
    cmd = bench.launch_command(["--gpus", "4", "--steps", "3"], 4, 29555)
    assert cmd[1:3] == ["-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd and "--master-addr=127.0.0.1" in cmd and "--master-port=29555" in cmd
    assert cmd[-4:] == ["--gpus", "4", "--steps", "3"] and cmd[-5].endswith("bench.py")
