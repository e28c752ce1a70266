"""Additions wider than one block: multi-block tiles chained by decoupled
look-back (bounded waits), against the oracle; failure injection on the host
side of the wait (a flag that nothing sets) reports MI_ETIMEOUT and leaves the
context usable."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import midint
import oracle as O
from carry_data import carry_stress

pytestmark = pytest.mark.gpu


@pytest.fixture
def wctx(lib):
    c = midint.Context(0)
    yield c
    c.close()


def run_add(c, devmem, a, b, m, limb_bits=64, six=False, offset=0):
    n = a.size // m
    words = a.view(np.uint32).size
    ba, pa = devmem.put(a, offset)
    bb, pb = devmem.put(b, offset)
    br, pr = devmem.empty_words(words, offset)
    dc = torch.full((n + 8,), 7, dtype=torch.uint8, device="cuda:0")
    s = torch.cuda.current_stream().cuda_stream
    if six:
        c.add6(pa, pb, pr, n, m, stream=s)
    else:
        c.add(pa, pb, pr, n, m, carry=dc.data_ptr(), limb_bits=limb_bits, stream=s)
    torch.cuda.synchronize()
    assert (br[offset + words:].cpu().numpy() == -1).all(), "result written past the batch"
    out = devmem.get(br, words, offset, a.dtype)
    cc = dc.cpu().numpy()
    assert (cc[n:] == 7).all()
    return out, cc[:n]


@pytest.mark.parametrize("m", [4097, 4607, 6144, 8192, 10000, 70001])
def test_wide_add_matches_oracle(wctx, devmem, m):
    n = 5 if m < 20000 else 2
    a, b = carry_stress(n, m, seed=m)
    r, c = run_add(wctx, devmem, a, b, m)
    ra, ca = O.add(a, b, m)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)
    assert wctx.device_status() == midint.MI_OK


def test_wide_add_carry_through_every_tile(wctx, devmem):
    # all-ones + 1 carries through every tile of the instance; all-ones + 0
    # propagates nowhere; a random instance in between
    m = 1 << 18
    a = np.full(3 * m, 0xFFFFFFFFFFFFFFFF, np.uint64)
    b = np.zeros(3 * m, np.uint64)
    b[0] = 1
    rng = np.random.default_rng(5)
    a[m:2 * m] = rng.integers(0, 2**64, m, dtype=np.uint64)
    b[m:2 * m] = rng.integers(0, 2**64, m, dtype=np.uint64)
    r, c = run_add(wctx, devmem, a, b, m)
    ra, ca = O.add(a, b, m)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)
    assert not r[:m].any() and c[0] == 1 and c[2] == 0


@pytest.mark.parametrize("m", [8193, 20001])
def test_wide_add_odd_u32(wctx, devmem, m):
    a, b = carry_stress(3, m, seed=m, dtype=np.uint32)
    r, c = run_add(wctx, devmem, a, b, m, limb_bits=32)
    ra, ca = O.add(a, b, m)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)


@pytest.mark.parametrize("m", [4100, 9000])
def test_wide_add6_matches_oracle(wctx, devmem, m):
    a, b = carry_stress(4, m, seed=m + 1)
    r, _ = run_add(wctx, devmem, a, b, m, six=True)
    assert np.array_equal(r, O.add6(a, b, m))


def test_wide_add_in_rounds(wctx, devmem):
    # 3 tiles per instance and 7 tiles per launch: 2 instances per round
    wctx.set_tuning(midint.TUNE_WIDE_ROUND_TILES, 0, 7)
    m = 5000
    a, b = carry_stress(9, m, seed=77)
    r, c = run_add(wctx, devmem, a, b, m)
    ra, ca = O.add(a, b, m)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)
    with pytest.raises(midint.MidintError):       # an instance needs 3 tiles
        wctx.set_tuning(midint.TUNE_WIDE_ROUND_TILES, 0, 2)
        run_add(wctx, devmem, a, b, m)


def test_wide_add_unaligned_rows(wctx, devmem):
    m = 4099
    a, b = carry_stress(3, m, seed=3)
    r, c = run_add(wctx, devmem, a.view(np.uint32), b.view(np.uint32), 2 * m, limb_bits=32, offset=1)
    ra, ca = O.add(a, b, m)
    assert np.array_equal(r.view(np.uint64), ra) and np.array_equal(c, ca)


def test_wide_add_timeout_is_reported_and_context_survives(wctx, devmem):
    m = 10000
    a, b = carry_stress(3, m, seed=11)
    wctx.set_tuning(midint.TUNE_WIDE_SPIN_LIMIT, 0, 256)
    wctx.set_tuning(midint.TUNE_WIDE_WITHHOLD, 0, 1)
    run_add(wctx, devmem, a, b, m)                # completes: the waits are bounded
    assert wctx.device_status() == midint.MI_ETIMEOUT
    assert wctx.device_status() == midint.MI_OK   # reading clears it
    # the host-buffer call reports it itself
    r = np.zeros_like(a)
    c = np.zeros(3, np.uint8)
    with pytest.raises(midint.MidintError):
        wctx.host_add(a, b, r, c, 3, m)
    # and the context is still good
    wctx.set_tuning(midint.TUNE_WIDE_WITHHOLD, 0, 0)
    wctx.set_tuning(midint.TUNE_WIDE_SPIN_LIMIT, 0, 1 << 20)
    rr, cc = run_add(wctx, devmem, a, b, m)
    ra, ca = O.add(a, b, m)
    assert np.array_equal(rr, ra) and np.array_equal(cc, ca)
    wctx.host_add(a, b, r, c, 3, m)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)
    assert wctx.device_status() == midint.MI_OK
