"""GPU addition vs the oracle, bit-exact, through the C ABI."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import midint
import oracle as O
from carry_data import carry_stress
from conftest import golden

pytestmark = pytest.mark.gpu


def _stream():
    return torch.cuda.current_stream().cuda_stream


def gpu_add(ctx, devmem, a, b, m, limb_bits=64, offset=0):
    n = a.size // m
    words = a.view(np.uint32).size
    ba, pa = devmem.put(a, offset)
    bb, pb = devmem.put(b, offset)
    br, pr = devmem.empty_words(words, offset)
    dc = torch.full((n + 8,), 7, dtype=torch.uint8, device="cuda:0")
    ctx.add(pa, pb, pr, n, m, carry=dc.data_ptr(), limb_bits=limb_bits, stream=_stream())
    torch.cuda.synchronize()
    r = devmem.get(br, words, offset, a.dtype)
    c = dc.cpu().numpy()
    assert (c[n:] == 7).all(), "carry written past the batch"
    assert (br[offset + words:].cpu().numpy() == -1).all(), "result written past the batch"
    return r, c[:n]


U64_SIZES = [1, 2, 3, 4, 5, 7, 8, 16, 31, 32, 33, 63, 64, 65, 100, 128, 129, 255, 256, 257, 1000, 1024, 2047, 4096]


@pytest.mark.parametrize("m", U64_SIZES)
@pytest.mark.parametrize("n", [1, 7, 300])
def test_add_u64_matches_oracle(ctx, devmem, m, n):
    if m * n > 2_000_000:
        pytest.skip("size")
    a, b = carry_stress(n, m, seed=1000 * m + n)
    r, c = gpu_add(ctx, devmem, a, b, m)
    wr, wc = O.add(a, b, m)
    assert np.array_equal(r, wr)
    assert np.array_equal(c, wc)


@pytest.mark.parametrize("m", [1, 3, 5, 9, 31, 127, 129, 255, 1023, 4097, 8191])
@pytest.mark.parametrize("offset", [0, 1])
def test_add_u32_odd_and_unaligned(ctx, devmem, m, offset):
    n = 37
    a, b = carry_stress(n, m, seed=m, dtype=np.uint32)
    r, c = gpu_add(ctx, devmem, a, b, m, limb_bits=32, offset=offset)
    wr, wc = O.add(a, b, m)
    assert np.array_equal(r, wr) and np.array_equal(c, wc)


@pytest.mark.parametrize("m", [2, 64, 128, 4096])
def test_add_u64_unaligned_rows(ctx, devmem, m):
    # 8-byte aligned but not 16-byte aligned buffers take the scalar path
    a, b = carry_stress(9, m, seed=5 + m)
    r, c = gpu_add(ctx, devmem, a, b, m, offset=2)
    r2, c2 = gpu_add(ctx, devmem, a, b, m, offset=6)
    wr, wc = O.add(a, b, m)
    assert np.array_equal(r, wr) and np.array_equal(c, wc)
    assert np.array_equal(r2, wr)


@pytest.mark.parametrize("m", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096])
def test_add_matches_reference_fixtures(ctx, devmem, m):
    g = golden("ref_sweep.npz")
    r, _ = gpu_add(ctx, devmem, g["a"], g["b"], m, limb_bits=32)
    assert np.array_equal(r, g[f"add_{m}"])
    w = golden("ref_worst.npz")
    r, c = gpu_add(ctx, devmem, w[f"wa_{m}"], w[f"wb_{m}"], m, limb_bits=32)
    assert np.array_equal(r, w[f"wadd_{m}"]) and c.all()


def test_add_config_shape_with_worst_case_rows(ctx, devmem):
    import workloads

    a, b = workloads.add_pairs(n=65536, m=64)
    r, c = gpu_add(ctx, devmem, a, b, 64)
    wr, wc = O.batch_u64("add", a, b, 64, threads=8)
    assert np.array_equal(r, wr) and np.array_equal(c, wc)
    assert c[::8].all() and not r.reshape(-1, 64)[::8].any()


def test_add_in_place(ctx, devmem):
    m, n = 64, 50
    a, b = carry_stress(n, m, seed=99)
    ba, pa = devmem.put(a)
    bb, pb = devmem.put(b)
    ctx.add(pa, pb, pa, n, m, stream=_stream())       # r aliases a exactly
    torch.cuda.synchronize()
    assert np.array_equal(devmem.get(ba, a.view(np.uint32).size), O.add(a, b, m, with_carry=False))


def test_add_empty_batch(ctx, devmem):
    ba, pa = devmem.put(np.zeros(8, np.uint64))
    ctx.add(pa, pa, pa, 0, 8, stream=_stream())


@pytest.mark.parametrize("m", [1, 2, 3, 4, 17, 33, 64, 65, 128, 1000, 2048, 4096])
def test_add6_matches_oracle(ctx, devmem, m):
    n = 41
    a, b = carry_stress(n, m, seed=7 * m)
    ba, pa = devmem.put(a)
    bb, pb = devmem.put(b)
    br, pr = devmem.empty_words(a.view(np.uint32).size)
    ctx.add6(pa, pb, pr, n, m, stream=_stream())
    torch.cuda.synchronize()
    assert np.array_equal(devmem.get(br, a.view(np.uint32).size), O.add6(a, b, m))


def test_compat_gpuAdd(lib):
    g = golden("ref_sweep.npz")
    for m in (16, 128, 4096):
        a, b = g["a"], g["b"]
        r = np.zeros_like(a)
        midint.gpuAdd(midint.U32bits, m, a.size // m, a, b, r)
        assert np.array_equal(r, g[f"add_{m}"])
        a64, b64 = a.view(np.uint64), b.view(np.uint64)
        r64 = np.zeros_like(a64)
        midint.gpuAdd(midint.U64bits, m // 2, a64.size // (m // 2), a64, b64, r64)
        assert np.array_equal(r64.view(np.uint32), g[f"add_{m}"])


def test_host_add_with_carry(ctx):
    a, b = carry_stress(1000, 64, seed=3)
    r = np.zeros_like(a)
    c = np.zeros(1000, np.uint8)
    ctx.host_add(a, b, r, c, 1000, 64)
    wr, wc = O.add(a, b, 64)
    assert np.array_equal(r, wr) and np.array_equal(c, wc)


@pytest.mark.parametrize("tb", [16, 32, 64])
@pytest.mark.parametrize("m", [1, 2, 3, 8, 17, 64, 65, 200, 1024, 2049, 4096])
def test_add_every_thread_width(lib, devmem, tb, m):
    """Every bytes-per-thread choice of the tuning table gives the same sums."""
    c = midint.Context(0)
    try:
        for cls in range(13):
            c.set_tuning(midint.TUNE_ADD_THREAD_BYTES, cls, tb)
        a, b = carry_stress(19, m, seed=5 * m + tb)
        ra, ca = O.add(a, b, m)
        r, cc = gpu_add(c, devmem, a, b, m)
        assert np.array_equal(r, ra) and np.array_equal(cc, ca)
        r6 = devmem.empty_words(a.view(np.uint32).size)
        ba, pa = devmem.put(a)
        bb, pb = devmem.put(b)
        c.add6(pa, pb, r6[1], 19, m, stream=_stream())
        torch.cuda.synchronize()
        assert np.array_equal(devmem.get(r6[0], a.view(np.uint32).size), O.add6(a, b, m))
        if m % 2 == 1:  # odd u32 limb counts take the scalar u32 kernel
            a32, b32 = a.view(np.uint32)[: 19 * m], b.view(np.uint32)[: 19 * m]
            r32, c32 = gpu_add(c, devmem, a32, b32, m, limb_bits=32)
            ref32, cref32 = O.add(a32, b32, m)
            assert np.array_equal(r32, ref32) and np.array_equal(c32, cref32)
    finally:
        c.close()


def test_tuning_rejects_bad_values(ctx):
    with pytest.raises(midint.MidintError):
        ctx.set_tuning(midint.TUNE_ADD_THREAD_BYTES, 13, 16)
    with pytest.raises(midint.MidintError):
        ctx.set_tuning(midint.TUNE_ADD_THREAD_BYTES, 3, 24)
    with pytest.raises(midint.MidintError):
        ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 0, 258)
    with pytest.raises(midint.MidintError):
        ctx.set_tuning(99, 0, 1)
    old = ctx.get_tuning(midint.TUNE_PLAIN_NTT_MIN)
    ctx.set_tuning(midint.TUNE_PLAIN_NTT_MIN, 0, 1025)
    assert ctx.get_tuning(midint.TUNE_PLAIN_NTT_MIN) == 1025
    ctx.set_tuning(midint.TUNE_PLAIN_NTT_MIN, 0, old)
