"""Host-buffer calls (mi_host_*): every chunking of the copy/compute pipeline
and the zero-copy path on mapped pinned buffers give the oracle's results."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import midint
import oracle as O
from carry_data import carry_stress

pytestmark = pytest.mark.gpu


def _pinned(x: np.ndarray) -> torch.Tensor:
    t = torch.from_numpy(x.view(np.int64) if x.dtype == np.uint64 else x).pin_memory()
    return t


@pytest.fixture
def hctx(lib):
    c = midint.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("chunks", [1, 3, 8, 64])
@pytest.mark.parametrize("pinned", [False, True])
def test_host_mul_full_chunkings(hctx, chunks, pinned):
    n, m = 1000, 64
    a, b = carry_stress(n, m, seed=chunks)
    hctx.set_tuning(midint.TUNE_HOST_CHUNKS, 1, chunks)
    hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 1, 0)
    want = O.mul(a, b, m, True)
    if pinned:
        pa, pb = _pinned(a), _pinned(b)
        pr = torch.zeros(2 * n * m, dtype=torch.int64).pin_memory()
        hctx.host_mul_full(pa, pb, pr, n, m)
        got = pr.numpy().view(np.uint64)
    else:
        got = np.zeros(2 * n * m, np.uint64)
        hctx.host_mul_full(a, b, got, n, m)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("chunks", [1, 5, 16])
def test_host_add_chunkings(hctx, chunks):
    n, m = 3001, 33
    a, b = carry_stress(n, m, seed=chunks + 100)
    hctx.set_tuning(midint.TUNE_HOST_CHUNKS, 0, chunks)
    hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 0, 0)
    r = np.zeros(n * m, np.uint64)
    c = np.zeros(n, np.uint8)
    hctx.host_add(a, b, r, c, n, m)
    ra, ca = O.add(a, b, m)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)


def test_zero_copy_on_pinned_buffers(hctx):
    hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 0, 1)
    hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 1, 1)
    n, m = 777, 128
    a, b = carry_stress(n, m, seed=9)
    pa, pb = _pinned(a), _pinned(b)
    pr = torch.zeros(2 * n * m, dtype=torch.int64).pin_memory()
    hctx.host_mul_full(pa, pb, pr, n, m)
    assert np.array_equal(pr.numpy().view(np.uint64), O.mul(a, b, m, True))
    na, ma = 2049, 64
    a, b = carry_stress(na, ma, seed=10)
    pa, pb = _pinned(a), _pinned(b)
    pr = torch.zeros(na * ma, dtype=torch.int64).pin_memory()
    pc = torch.zeros(na, dtype=torch.uint8).pin_memory()
    hctx.host_add(pa, pb, pr, pc, na, ma)
    ra, ca = O.add(a, b, ma)
    assert np.array_equal(pr.numpy().view(np.uint64), ra) and np.array_equal(pc.numpy(), ca)
    # pageable buffers fall back to the copy pipeline
    r = np.zeros(na * ma, np.uint64)
    c = np.zeros(na, np.uint8)
    hctx.host_add(a, b, r, c, na, ma)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)


@pytest.mark.parametrize("chunks", [1, 3, 8])
@pytest.mark.parametrize("pinned", [False, True])
def test_copied_operands_with_results_in_place(hctx, chunks, pinned):
    """Mode 3: operands copied in by chunks, results written in place."""
    for cls in (0, 1):
        hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, cls, 3)
        hctx.set_tuning(midint.TUNE_HOST_CHUNKS, cls, chunks)
    n, m = 515, 64
    a, b = carry_stress(n, m, seed=chunks + 31)
    if pinned:
        pr = torch.zeros(2 * n * m, dtype=torch.int64).pin_memory()
        hctx.host_mul_full(_pinned(a), _pinned(b), pr, n, m)
        got = pr.numpy().view(np.uint64)
    else:  # pageable results: the copy pipeline
        got = np.zeros(2 * n * m, np.uint64)
        hctx.host_mul_full(a, b, got, n, m)
    assert np.array_equal(got, O.mul(a, b, m, True))
    ra, ca = O.add(a, b, m)
    if pinned:
        pr = torch.zeros(n * m, dtype=torch.int64).pin_memory()
        pc = torch.zeros(n, dtype=torch.uint8).pin_memory()
        hctx.host_add(a, b, pr, pc, n, m)
        r, c = pr.numpy().view(np.uint64), pc.numpy()
    else:
        r, c = np.zeros(n * m, np.uint64), np.zeros(n, np.uint8)
        hctx.host_add(a, b, r, c, n, m)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)
    # a wide addition with its results in place
    mw = 5000
    aw, bw = carry_stress(3, mw, seed=4)
    rw = torch.zeros(3 * mw, dtype=torch.int64).pin_memory()
    cw = torch.zeros(3, dtype=torch.uint8).pin_memory()
    hctx.host_add(aw, bw, rw, cw, 3, mw)
    raw, caw = O.add(aw, bw, mw)
    assert np.array_equal(rw.numpy().view(np.uint64), raw) and np.array_equal(cw.numpy(), caw)


@pytest.mark.parametrize("blocks", [1, 2, 3])
def test_zero_copy_with_capped_occupancy(hctx, blocks):
    """Mode 1 with the product kernel held to 1..3 resident blocks per SM."""
    hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 1, 1)
    hctx.set_tuning(midint.TUNE_HOST_ZC_BLOCKS, 1, blocks)
    assert hctx.get_tuning(midint.TUNE_HOST_ZC_BLOCKS, 1) == blocks
    for n, m in ((1500, 128), (999, 64), (37, 5), (64, 512)):
        a, b = carry_stress(n, m, seed=blocks * 100 + m)
        pa, pb = _pinned(a), _pinned(b)
        pr = torch.zeros(2 * n * m, dtype=torch.int64).pin_memory()
        hctx.host_mul_full(pa, pb, pr, n, m)
        assert np.array_equal(pr.numpy().view(np.uint64), O.mul(a, b, m, True))
    hctx.set_tuning(midint.TUNE_HOST_ZC_BLOCKS, 1, 0)


@pytest.mark.parametrize("m", [64, 128])
def test_zero_copy_strides_over_a_large_batch(hctx, m):
    """Mode 1 on a batch larger than the capped grid (32 blocks per SM of
    256 threads): each group reads its next instance's operands while it
    multiplies the current one, over several rounds and a ragged last one."""
    hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 1, 1)
    hctx.set_tuning(midint.TUNE_HOST_ZC_BLOCKS, 1, 2)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    per_block = 256 // (m // 4)  # instances of one 256-thread block (groups of m/4 threads)
    n = sms * 32 * per_block + 777
    a, b = carry_stress(n, m, seed=m + 5)
    pa, pb = _pinned(a), _pinned(b)
    pr = torch.zeros(2 * n * m, dtype=torch.int64).pin_memory()
    hctx.host_mul_full(pa, pb, pr, n, m)
    assert np.array_equal(pr.numpy().view(np.uint64), O.mul(a, b, m, True))
    hctx.set_tuning(midint.TUNE_HOST_ZC_BLOCKS, 1, 0)


@pytest.mark.parametrize("chunks", [1, 3, 8])
@pytest.mark.parametrize("pinned_out", [False, True])
def test_zero_copy_reads_with_copied_results(hctx, chunks, pinned_out):
    """Mode 2: operands read in place, results copied out in chunks."""
    for cls in (0, 1):
        hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, cls, 2)
        hctx.set_tuning(midint.TUNE_HOST_CHUNKS, cls, chunks)
    n, m = 513, 64
    a, b = carry_stress(n, m, seed=chunks + 7)
    pa, pb = _pinned(a), _pinned(b)
    if pinned_out:
        pr = torch.zeros(2 * n * m, dtype=torch.int64).pin_memory()
        hctx.host_mul_full(pa, pb, pr, n, m)
        got = pr.numpy().view(np.uint64)
    else:
        got = np.zeros(2 * n * m, np.uint64)
        hctx.host_mul_full(pa, pb, got, n, m)
    assert np.array_equal(got, O.mul(a, b, m, True))
    r = np.zeros(n * m, np.uint64)
    c = np.zeros(n, np.uint8)
    hctx.host_add(pa, pb, r, c, n, m)
    ra, ca = O.add(a, b, m)
    assert np.array_equal(r, ra) and np.array_equal(c, ca)
    # a wide addition in this mode keeps its launches on one stream
    mw = 5000
    aw, bw = carry_stress(3, mw, seed=2)
    rw = np.zeros(3 * mw, np.uint64)
    cw = np.zeros(3, np.uint8)
    hctx.host_add(_pinned(aw), _pinned(bw), rw, cw, 3, mw)
    raw, caw = O.add(aw, bw, mw)
    assert np.array_equal(rw, raw) and np.array_equal(cw, caw)


def test_host_tuning_knobs_are_checked(hctx):
    with pytest.raises(midint.MidintError):
        hctx.set_tuning(midint.TUNE_HOST_CHUNKS, 0, 0)
    with pytest.raises(midint.MidintError):
        hctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 0, 4)
    with pytest.raises(midint.MidintError):
        hctx.set_tuning(midint.TUNE_HOST_CHUNKS, 2, 4)
    with pytest.raises(midint.MidintError):
        hctx.set_tuning(midint.TUNE_HOST_ZC_BLOCKS, 1, 4)
    with pytest.raises(midint.MidintError):
        hctx.set_tuning(midint.TUNE_HOST_ZC_BLOCKS, 2, 1)
    hctx.set_tuning(midint.TUNE_HOST_CHUNKS, 1, 5)
    assert hctx.get_tuning(midint.TUNE_HOST_CHUNKS, 1) == 5


@pytest.mark.parametrize("m", [320, 512, 2048])
def test_compat_gpuMultiply_ntt_low_half_on_pinned_buffers(lib, m):
    """The u64 gpuMultiply wrapper takes the NTT low half from 320 limbs on;
    on mapped pinned buffers its kernel reads and writes them in place (the
    tuned zero-copy mode of products), on pageable ones through copies."""
    n = 40
    a, b = carry_stress(n, m, seed=m + 3)
    want = O.mul(a, b, m, False)
    pa, pb = _pinned(a), _pinned(b)
    pr = torch.zeros(n * m, dtype=torch.int64).pin_memory()
    midint.check(lib.mi_compat_gpuMultiply_u64(n, m, pa.data_ptr(), pb.data_ptr(), pr.data_ptr()))
    assert np.array_equal(pr.numpy().view(np.uint64), want)
    r = np.zeros(n * m, np.uint64)
    midint.gpuMultiply(midint.U64bits, m, n, a, b, r)
    assert np.array_equal(r, want)


def test_contexts_on_several_host_threads(lib):
    """Host threads with their own contexts and different zero-copy occupancy
    caps (different shared-memory requests of the same product kernel) call
    at once; every result is the oracle's."""
    import threading

    n, m = 600, 128
    a, b = carry_stress(n, m, seed=404)
    want = O.mul(a, b, m, True)
    pa, pb = _pinned(a), _pinned(b)
    outs = [torch.zeros(2 * n * m, dtype=torch.int64).pin_memory() for _ in range(4)]
    ctxs = [midint.Context(0) for _ in range(4)]
    errors = []
    start = threading.Barrier(4)

    def run(i):
        try:
            ctxs[i].set_tuning(midint.TUNE_HOST_ZERO_COPY, 1, 1)
            ctxs[i].set_tuning(midint.TUNE_HOST_ZC_BLOCKS, 1, i)
            start.wait()
            for _ in range(3):
                ctxs[i].host_mul_full(pa, pb, outs[i], n, m)
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for c in ctxs:
        c.close()
    assert not errors, errors
    for o in outs:
        assert np.array_equal(o.numpy().view(np.uint64), want)


def test_calib_host_link(ctx):
    # SM-driven streaming over mapped pinned memory: plausible rates, and
    # sizes that are not a multiple of 32 bytes refused before any launch
    nb = 8 << 20
    src = torch.empty(nb, dtype=torch.uint8).pin_memory()
    dst = torch.empty(nb, dtype=torch.uint8).pin_memory()
    r, w, b = midint.calib_host_link(src, dst, nb)
    assert 1.0 < r < 5000.0 and 1.0 < w < 5000.0 and 1.0 < b < 10000.0
    with pytest.raises(midint.MidintError) as e:
        midint.calib_host_link(src, dst, nb - 16)
    assert e.value.status == midint.MI_EINVAL
