"""The synthetic workloads on CPU: seeded and reproducible, the documented
shapes and worst-case fractions, and ragged lists whose operand and result
ranges tile their pools exactly (what the ragged kernels index)."""
from __future__ import annotations

import numpy as np

import midint
import workloads


def test_splitmix64_is_seeded():
    a = workloads.splitmix64(123, 1000)
    assert a.dtype == np.uint64 and a.size == 1000
    assert np.array_equal(a, workloads.splitmix64(123, 1000))
    assert not np.array_equal(a, workloads.splitmix64(124, 1000))
    assert np.array_equal(workloads.splitmix64(123, 10), a[:10])


def test_add_pairs_worst_case_fraction():
    n, m = 4096, 16
    a, b = workloads.add_pairs(n=n, m=m)
    assert a.size == b.size == n * m
    full = np.uint64(0xFFFFFFFFFFFFFFFF)
    rows_a, rows_b = a.reshape(n, m), b.reshape(n, m)
    worst = np.all(rows_a == full, axis=1)
    assert worst.sum() == n // 8
    assert np.array_equal(np.flatnonzero(worst) % 8, np.zeros(n // 8, int))
    # each all-ones row meets 1: the carry runs through every limb and out
    one = np.zeros(m, np.uint64)
    one[0] = 1
    assert all(np.array_equal(r, one) for r in rows_b[worst])


def test_ntt_pairs_all_ones_fraction():
    n, m = 256, 8
    a, b = workloads.ntt_pairs(n=n, m=m)
    full = np.uint64(0xFFFFFFFFFFFFFFFF)
    ones = np.all(a.reshape(n, m) == full, axis=1) & np.all(b.reshape(n, m) == full, axis=1)
    assert ones.sum() == n // 16


def test_ragged_ops_tile_their_pools():
    ops, pool, out_limbs = workloads.ragged_ops(n_ops=5000)
    assert ops.dtype.itemsize == np.dtype(midint.OP_DTYPE).itemsize
    la, lb = ops["la"].astype(np.uint64), ops["lb"].astype(np.uint64)
    assert ops["la"].min() >= 4 and ops["la"].max() <= 1024 and ops["lb"].min() >= 4
    # operands: a_i then b_i, back to back, covering the pool exactly
    assert ops["a_off"][0] == 0
    assert np.array_equal(ops["b_off"], ops["a_off"] + la)
    assert np.array_equal(ops["a_off"][1:], ops["b_off"][:-1] + lb[:-1])
    assert int(ops["b_off"][-1] + lb[-1]) == pool.size
    # results: max(la, lb) limbs per add, la + lb per product, in op order
    rlen = np.where(ops["kind"] == 0, np.maximum(la, lb), la + lb)
    assert np.array_equal(ops["r_off"][1:], ops["r_off"][:-1] + rlen[:-1])
    assert int(ops["r_off"][-1] + rlen[-1]) == out_limbs
    frac_add = float((ops["kind"] == 0).mean())
    assert 0.37 < frac_add < 0.43
    again, pool2, _ = workloads.ragged_ops(n_ops=5000)
    assert np.array_equal(again, ops) and np.array_equal(pool2, pool)
