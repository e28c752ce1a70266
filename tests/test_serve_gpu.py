"""The request loop: every result is bit-identical whether the request runs
alone or in a mix of concurrently admitted requests, in both the
continuous-batching and the per-request mode, and matches the oracle."""
from __future__ import annotations

import numpy as np
import pytest

import midint
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu


def make_request(seed, n_ops=None):
    rng = np.random.default_rng(seed)
    n = int(n_ops or rng.integers(1, 513))
    kind = rng.integers(0, 2, n).astype(np.uint32)
    lo, hi = np.log(512), np.log(32768)
    la = np.ceil(np.exp(rng.uniform(lo, hi, n)) / 64).astype(np.uint32)
    lb = np.ceil(np.exp(rng.uniform(lo, hi, n)) / 64).astype(np.uint32)
    ops, pool, out_limbs = W.pack_ops(kind, la, lb, seed)
    return ops, pool, out_limbs


def check_against_oracle(ops, pool, out, carry, sample):
    for i in sample:
        op = ops[i]
        la, lb = int(op["la"]), int(op["lb"])
        m = max(la, lb)
        aa = np.zeros(m, np.uint64); aa[:la] = pool[int(op["a_off"]):int(op["a_off"]) + la]
        bb = np.zeros(m, np.uint64); bb[:lb] = pool[int(op["b_off"]):int(op["b_off"]) + lb]
        ro = int(op["r_off"])
        if op["kind"] == 0:
            want, wc = O.add(aa, bb, m)
            assert np.array_equal(out[ro:ro + m], want) and carry[i] == wc[0]
        else:
            assert np.array_equal(out[ro:ro + la + lb], O.mul(aa, bb, m, True)[:la + lb])


def run_alone(ctx, req, batching):
    ops, pool, out_limbs = req
    out = np.zeros(out_limbs, np.uint64)
    carry = np.zeros(ops.size, np.uint8)
    with midint.Server(ctx, device_bytes=256 << 20, slots=2, batching=batching) as srv:
        t = srv.submit(ops, pool, out, carry)
        srv.wait(t, 60000)
    return out, carry


@pytest.mark.parametrize("batching", [True, False])
def test_each_result_is_the_same_alone_and_in_the_mix(ctx, batching):
    reqs = [make_request(100 + i) for i in range(24)]
    outs = [np.zeros(r[2], np.uint64) for r in reqs]
    carries = [np.zeros(r[0].size, np.uint8) for r in reqs]
    # small arenas force many batches, several of them in flight at once
    with midint.Server(ctx, device_bytes=64 << 20, slots=3, batching=batching) as srv:
        tickets = [srv.submit(r[0], r[1], o, c) for r, o, c in zip(reqs, outs, carries)]
        for t in tickets:
            srv.wait(t, 120000)
        batches, done, n_ops = srv.stats()
        assert done == len(reqs) and n_ops == sum(r[0].size for r in reqs)
        if batching:
            assert batches < len(reqs)      # requests were admitted together
        else:
            assert batches == len(reqs)     # one request per launch
        times = [srv.times(t) for t in tickets]
    assert all(s <= a <= d for s, a, d in times)
    for i in (0, 5, 11, 23):
        alone_out, alone_carry = run_alone(ctx, reqs[i], batching=True)
        assert np.array_equal(alone_out, outs[i])
        adds = reqs[i][0]["kind"] == 0
        assert np.array_equal(alone_carry[adds], carries[i][adds])
    for i in (0, 7, 23):
        ops, pool, _ = reqs[i]
        check_against_oracle(ops, pool, outs[i], carries[i], range(0, ops.size, max(1, ops.size // 20)))


def test_single_large_request_grows_the_arena(ctx):
    req = make_request(7, n_ops=512)
    out = np.zeros(req[2], np.uint64)
    carry = np.zeros(req[0].size, np.uint8)
    with midint.Server(ctx, device_bytes=1 << 20, slots=1) as srv:   # arena smaller than the request
        t = srv.submit(req[0], req[1], out, carry)
        srv.wait(t, 60000)
    check_against_oracle(req[0], req[1], out, carry, range(0, 512, 37))


def test_malformed_requests_are_refused(ctx):
    ops, pool, out_limbs = make_request(3, n_ops=4)
    out = np.zeros(out_limbs, np.uint64)
    with midint.Server(ctx, device_bytes=16 << 20, slots=1) as srv:
        bad = ops.copy()
        bad["a_off"][2] = pool.size        # operand outside the request's pool
        with pytest.raises(midint.MidintError) as e:
            srv.submit(bad, pool, out)
        assert e.value.status == midint.MI_EINVAL
        with pytest.raises(midint.MidintError):
            srv.wait(12345, 0)             # unknown ticket
