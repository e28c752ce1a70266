"""Dependent calls back to back on one stream with no synchronisation between
them: every call reads what the one before it wrote.

The plain-path kernels are launched with programmatic stream serialisation:
their blocks may become resident while the previous kernel of the stream is
still running, and wait for it before their first memory access.  These
chains check that each call still sees the complete result of its
predecessor, across every kernel family and across a large producer followed
by a small consumer (whose blocks are all resident long before the producer
ends).
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu


def _rand(rng, n):
    return rng.integers(0, 2**64, n, dtype=np.uint64)


def _dev(x):
    return torch.from_numpy(x.view(np.int64).copy()).to("cuda:0")


def _host(t):
    return t.cpu().numpy().view(np.uint64)


def test_dependent_chain_matches_oracle(ctx):
    rng = np.random.default_rng(2024)
    n, m = 4096, 64
    a, b, c = _rand(rng, n * m), _rand(rng, n * m), _rand(rng, n * m)
    a[: 8 * m] = np.uint64(2**64 - 1)  # carries through whole instances
    b[: 8 * m] = 0
    b[: 8 * m: m] = 1
    da, db, dc = _dev(a), _dev(b), _dev(c)
    ds, dl, dq, du, dv = (torch.empty(n * m, dtype=torch.int64, device="cuda:0") for _ in range(5))
    dw = torch.empty(n * m * 2, dtype=torch.int32, device="cuda:0")  # 4-byte words
    dp = torch.empty(2 * n * m, dtype=torch.int64, device="cuda:0")
    dn = torch.empty(2 * n * m, dtype=torch.int64, device="cuda:0")
    st = torch.cuda.current_stream().cuda_stream
    rounds = 3
    for _ in range(rounds):
        ctx.add(da, db, ds, n, m, stream=st)                       # s = a + b
        ctx.mul_lo(ds, dc, dl, n, m, stream=st)                    # l = s * c mod 2^(64m)
        ctx.poly(dl, ds, dq, n, m, stream=st)                      # q = poly(l, s)
        ctx.add6(dq, dl, du, n, m, stream=st)                      # u = 6q + 10l
        ctx.export_words(du, n, m, dw, 2 * m, 4, 1, 1, stream=st)  # big-endian words, most significant first
        ctx.import_words(dw, n, 2 * m, 4, 1, 1, dv, m, stream=st)  # and back: v = u
        ctx.mul_full(dv, da, dp, n, m, stream=st)                  # p = v * a
        ctx.mul_ntt(dv, da, dn, n, m, stream=st)                   # the same by NTT
        ctx.add(dv, ds, da, n, m, stream=st)                       # next round's a = v + s
    torch.cuda.synchronize()
    for _ in range(rounds):
        s = O.add(a, b, m)[0]
        l = O.mul(s, c, m, False)
        q = O.poly(l, s, m)
        u = O.add6(q, l, m)
        p = O.mul(u, a, m, True)
        a = O.add(u, s, m)[0]
    assert np.array_equal(_host(dp), p)
    assert np.array_equal(_host(dn), p)
    assert np.array_equal(_host(da), a)


def test_large_producer_small_consumer(ctx):
    """A long addition, then a one-instance product of its last instance."""
    rng = np.random.default_rng(7)
    n, m = 262144, 64
    a, b = _rand(rng, n * m), _rand(rng, n * m)
    da, db = _dev(a), _dev(b)
    ds = torch.empty(n * m, dtype=torch.int64, device="cuda:0")
    dp = torch.empty(2 * m, dtype=torch.int64, device="cuda:0")
    st = torch.cuda.current_stream().cuda_stream
    last = ds[(n - 1) * m:]
    for _ in range(4):
        ctx.add(da, db, ds, n, m, stream=st)
        ctx.mul_full(last, last, dp, 1, m, stream=st)
        ctx.add(ds, db, da, n, m, stream=st)  # overwrite a: the next product must see the new sum
    torch.cuda.synchronize()
    for _ in range(4):
        s = O.add(a, b, m)[0]
        p = O.mul(s[(n - 1) * m:], s[(n - 1) * m:], m, True)
        a = O.add(s, b, m)[0]
    assert np.array_equal(_host(dp), p)
    assert np.array_equal(_host(da), a)
