"""mi_ragged_run_noalloc: the ragged run for callers that cannot allocate
device memory (code inside another framework's memory pool or under a fixed
device budget).  It must give exactly what mi_ragged_run gives with a caller
scratch buffer, on consecutive calls that share its static scratch.

Collected last on purpose (file name), so that a failure here comes after
every other test has run; it also passes alone in a fresh process."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import midint
import workloads as W

pytestmark = pytest.mark.gpu


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _device_inputs(ops, pool, out_limbs):
    d_ops = torch.from_numpy(ops.view(np.uint8).copy()).to("cuda:0")
    d_in = torch.from_numpy(pool.view(np.int64)).to("cuda:0")
    d_out = torch.full((out_limbs,), -1, dtype=torch.int64, device="cuda:0")
    d_c = torch.full((ops.size,), 7, dtype=torch.uint8, device="cuda:0")
    return d_ops, d_in, d_out, d_c


def with_scratch(ctx, ops, pool, out_limbs):
    d_ops, d_in, d_out, d_c = _device_inputs(ops, pool, out_limbs)
    sb = midint.ragged_scratch_bytes(ops.size)
    scr = torch.empty(sb // 4 + 1, dtype=torch.int32, device="cuda:0")
    ctx.ragged_run(d_ops, ops.size, d_in, d_out, scr, sb, carry=d_c, stream=_stream())
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint64), d_c.cpu().numpy()


def without_scratch(ctx, ops, pool, out_limbs):
    d_ops, d_in, d_out, d_c = _device_inputs(ops, pool, out_limbs)
    ctx.ragged_run_noalloc(d_ops, ops.size, d_in, d_out, carry=d_c, stream=_stream())
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint64), d_c.cpu().numpy()


def test_noalloc_matches_scratch_entry_point_on_two_calls_in_a_row(ctx):
    # two different lists back to back: the second call reuses the static
    # scratch with the first call's contents still in it
    first = W.ragged_ops(n_ops=6000, seed=21)
    second = W.ragged_ops(n_ops=2500, seed=22)
    for ops, pool, out_limbs in (first, second):
        got_out, got_c = without_scratch(ctx, ops, pool, out_limbs)
        want_out, want_c = with_scratch(ctx, ops, pool, out_limbs)
        assert np.array_equal(got_out, want_out)
        adds = ops["kind"] == 0
        assert np.array_equal(got_c[adds], want_c[adds])


def test_noalloc_at_its_static_limit(ctx):
    # exactly as many ops as the static array is sized for
    ops, pool, out_limbs = W.ragged_ops(n_ops=midint.RAGGED_NOALLOC_MAX_OPS, seed=23)
    got_out, got_c = without_scratch(ctx, ops, pool, out_limbs)
    assert ctx.ragged_invalid_noalloc() == 0
    want_out, want_c = with_scratch(ctx, ops, pool, out_limbs)
    assert np.array_equal(got_out, want_out)
    adds = ops["kind"] == 0
    assert np.array_equal(got_c[adds], want_c[adds])


def test_noalloc_counts_invalid_ops(ctx):
    # a bad kind, a zero length and an over-long operand are skipped and counted
    ops, pool, out_limbs = W.pack_ops(np.array([0, 1, 1, 0, 7], np.uint32), np.array([3, 5, 0, 2000, 4], np.uint32),
                                      np.array([3, 6, 4, 3, 4], np.uint32), 3)
    got_out, got_c = without_scratch(ctx, ops, pool, out_limbs)
    assert ctx.ragged_invalid_noalloc() == 3
    want_out, want_c = with_scratch(ctx, ops, pool, out_limbs)
    assert np.array_equal(got_out, want_out) and got_c[0] == want_c[0]


def test_noalloc_refuses_lists_beyond_its_static_scratch(ctx):
    n = midint.RAGGED_NOALLOC_MAX_OPS + 1
    dummy = torch.zeros(8, dtype=torch.int64, device="cuda:0")
    with pytest.raises(midint.MidintError) as e:
        ctx.ragged_run_noalloc(dummy, n, dummy, dummy, stream=_stream())
    assert e.value.status == midint.MI_EINVAL
    assert "static scratch" in e.value.detail
