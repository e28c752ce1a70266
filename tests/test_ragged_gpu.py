"""Ragged batches on the GPU vs the oracle (bit-exact), the plain per-class
form vs the ragged kernels, invalid ops, and CUDA-graph replay."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import midint
import oracle as O
import workloads as W
from plainform import PlainBatch

pytestmark = pytest.mark.gpu

EDGE = [1, 2, 3, 4, 5, 8, 15, 16, 17, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129, 200, 255, 256, 257,
        400, 511, 512, 513, 700, 1000, 1023, 1024]


def _stream():
    return torch.cuda.current_stream().cuda_stream


def run_ragged(ctx, ops, pool, out_limbs, graph=False, replays=1):
    n = ops.size
    d_ops = torch.from_numpy(ops.view(np.uint8).copy()).to("cuda:0")
    d_in = torch.from_numpy(pool.view(np.int64)).to("cuda:0")
    d_out = torch.full((out_limbs + 16,), -1, dtype=torch.int64, device="cuda:0")
    d_c = torch.full((n + 16,), 7, dtype=torch.uint8, device="cuda:0")
    sb = midint.ragged_scratch_bytes(n)
    scr = torch.empty(sb // 4 + 1, dtype=torch.int32, device="cuda:0")
    if graph:
        g = ctx.ragged_graph(d_ops, n, d_in, d_out, scr, sb, carry=d_c)
        for _ in range(replays):
            g.launch(_stream())
        torch.cuda.synchronize()
        g.close()
    else:
        for _ in range(replays):
            ctx.ragged_run(d_ops, n, d_in, d_out, scr, sb, carry=d_c, stream=_stream())
        torch.cuda.synchronize()
    out = d_out.cpu().numpy().view(np.uint64)
    assert (out[out_limbs:] == np.uint64(2**64 - 1)).all(), "write past the output pool"
    carry = d_c.cpu().numpy()
    assert (carry[n:] == 7).all()
    return out[:out_limbs], carry[:n], midint.ragged_invalid(scr)


def oracle_check(ops, pool, out, carry, sample=None):
    idx = range(ops.size) if sample is None else sample
    for i in idx:
        op = ops[i]
        la, lb = int(op["la"]), int(op["lb"])
        a = pool[int(op["a_off"]):int(op["a_off"]) + la]
        b = pool[int(op["b_off"]):int(op["b_off"]) + lb]
        ro = int(op["r_off"])
        if op["kind"] == 0:
            m = max(la, lb)
            aa = np.zeros(m, np.uint64); aa[:la] = a
            bb = np.zeros(m, np.uint64); bb[:lb] = b
            want, wc = O.add(aa, bb, m)
            assert np.array_equal(out[ro:ro + m], want), f"add op {i} ({la}, {lb})"
            assert carry[i] == wc[0], f"add carry op {i}"
        else:
            m = max(la, lb)
            aa = np.zeros(m, np.uint64); aa[:la] = a
            bb = np.zeros(m, np.uint64); bb[:lb] = b
            want = O.mul(aa, bb, m, True)[:la + lb]
            assert np.array_equal(out[ro:ro + la + lb], want), f"mul op {i} ({la}, {lb})"


def edge_ops(seed, n_rand=600):
    rng = np.random.default_rng(seed)
    la, lb, kind = [], [], []
    for k in (0, 1):
        for x in EDGE:
            for y in (1, 4, 64, 128, 129, 200, 256, 257, 1024, x):
                la.append(x); lb.append(y); kind.append(k)
                la.append(y); lb.append(x); kind.append(k)
    la += list(rng.integers(1, 1025, n_rand)); lb += list(rng.integers(1, 1025, n_rand))
    kind += list(rng.integers(0, 2, n_rand))
    return W.pack_ops(np.array(kind, np.uint32), np.array(la, np.uint32), np.array(lb, np.uint32), seed)


# (ntt_min, ntt40_min): the shorter operand from which every product takes
# the NTT, and from which products whose NTT runs on 40-bit digits do
@pytest.mark.parametrize("ntt_min,ntt40_min", [(257, 257), (257, 1), (200, 64), (129, 129), (128, 80), (64, 64),
                                               (1, 1)])
def test_ragged_matches_oracle(ctx, ntt_min, ntt40_min):
    ops, pool, out_limbs = edge_ops(seed=ntt_min + ntt40_min)
    # worst-case carries for some adds: a all ones, b = 1
    for i in range(0, ops.size, 7):
        if ops["kind"][i] == 0:
            ao, la = int(ops["a_off"][i]), int(ops["la"][i])
            bo, lb = int(ops["b_off"][i]), int(ops["lb"][i])
            pool[ao:ao + la] = np.uint64(2**64 - 1)
            pool[bo:bo + lb] = 0
            pool[bo] = 1
    old = ctx.get_tuning(midint.TUNE_RAGGED_NTT_MIN), ctx.get_tuning(midint.TUNE_RAGGED_NTT_MIN, 1)
    ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 0, ntt_min)
    ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 1, ntt40_min)
    try:
        out, carry, invalid = run_ragged(ctx, ops, pool, out_limbs)
    finally:
        ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 0, old[0])
        ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 1, old[1])
    assert invalid == 0
    oracle_check(ops, pool, out, carry)


def test_ragged_all_ones_products(ctx):
    # 300 x 300, 525 x 525 and 525 x 700 run on 40-bit digits and three primes
    # (525 limbs: the largest shorter operand they keep exact), 526 x 526 on
    # 48-bit digits and four
    kind = np.ones(56, np.uint32)
    la = np.array([1024, 1000, 129, 128, 64, 7, 1024, 300, 256, 257, 525, 525, 526, 160] * 4, np.uint32)
    lb = np.array([1024, 3, 128, 129, 1024, 1024, 1, 300, 1024, 200, 525, 700, 526, 160] * 4, np.uint32)
    ops, pool, out_limbs = W.pack_ops(kind, la, lb, 9)
    pool[:] = np.uint64(2**64 - 1)
    old = ctx.get_tuning(midint.TUNE_RAGGED_NTT_MIN)
    old40 = ctx.get_tuning(midint.TUNE_RAGGED_NTT_MIN, 1)
    for ntt_min, ntt40_min in ((257, 257), (200, 200), (129, 129), (257, 1), (1, 1)):
        ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 0, ntt_min)
        ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 1, ntt40_min)
        out, carry, _ = run_ragged(ctx, ops, pool, out_limbs)
        oracle_check(ops, pool, out, carry)
    ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 0, old)
    ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 1, old40)


def test_ragged_invalid_ops_are_skipped(ctx):
    ops, pool, out_limbs = W.pack_ops(np.array([0, 1, 1, 0, 7], np.uint32), np.array([3, 5, 0, 2000, 4], np.uint32),
                                      np.array([3, 6, 4, 3, 4], np.uint32), 3)
    out, carry, invalid = run_ragged(ctx, ops, pool, out_limbs)
    assert invalid == 3
    oracle_check(ops, pool, out, carry, sample=[0, 1])


def test_ragged_rejects_misaligned_pools(ctx):
    ops, pool, out_limbs = W.ragged_ops(n_ops=10, seed=4)
    d_ops = torch.from_numpy(ops.view(np.uint8).copy()).to("cuda:0")
    d_in = torch.from_numpy(pool.view(np.int64)).to("cuda:0")
    d_out = torch.zeros(out_limbs + 1, dtype=torch.int64, device="cuda:0")
    sb = midint.ragged_scratch_bytes(ops.size)
    scr = torch.empty(sb // 4 + 1, dtype=torch.int32, device="cuda:0")
    with pytest.raises(midint.MidintError) as e:
        ctx.ragged_run(d_ops, ops.size, d_in, d_out.data_ptr() + 4, scr, sb, stream=_stream())
    assert e.value.status == midint.MI_EINVAL
    with pytest.raises(midint.MidintError):
        ctx.ragged_run_noalloc(d_ops, ops.size, d_in.data_ptr() + 4, d_out, stream=_stream())


def test_ragged_graph_replay_matches_direct_run(ctx):
    ops, pool, out_limbs = W.ragged_ops(n_ops=5000, seed=11)
    direct, c1, _ = run_ragged(ctx, ops, pool, out_limbs)
    replayed, c2, _ = run_ragged(ctx, ops, pool, out_limbs, graph=True, replays=3)
    assert np.array_equal(direct, replayed) and np.array_equal(c1, c2)
    oracle_check(ops, pool, direct, c1, sample=range(0, 5000, 17))


def test_ragged_full_workload_matches_plain_form(ctx):
    ops, pool, out_limbs = W.ragged_ops()
    out, carry, invalid = run_ragged(ctx, ops, pool, out_limbs)
    assert invalid == 0
    plain = PlainBatch(ops, pool)
    plain.run(ctx, _stream())
    torch.cuda.synchronize()
    p_out, p_carry = plain.results(ops, out_limbs)
    assert np.array_equal(out, p_out)
    adds = ops["kind"] == 0
    assert np.array_equal(carry[adds], p_carry[adds])
    oracle_check(ops, pool, out, carry, sample=range(0, ops.size, 997))
