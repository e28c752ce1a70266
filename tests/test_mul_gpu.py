"""GPU classical multiplication vs the oracle, bit-exact, through the C ABI."""
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


def gpu_mul(ctx, devmem, a, b, m, full=True, limb_bits=64, offset=0):
    n = a.size // m
    in_words = a.view(np.uint32).size
    out_words = in_words * (2 if full else 1)
    ba, pa = devmem.put(a, offset)
    bb, pb = devmem.put(b, offset)
    br, pr = devmem.empty_words(out_words, offset)
    f = ctx.mul_full if full else ctx.mul_lo
    f(pa, pb, pr, n, m, limb_bits=limb_bits, stream=_stream())
    torch.cuda.synchronize()
    assert (br[offset + out_words:].cpu().numpy() == -1).all(), "result written past the batch"
    return devmem.get(br, out_words, offset, a.dtype)


U64_SIZES = [1, 2, 3, 4, 5, 8, 15, 16, 17, 31, 32, 33, 64, 100, 128, 129, 200, 256, 500, 512, 1000, 1024, 1025,
             1500, 2047, 2048]


@pytest.mark.parametrize("m", U64_SIZES)
@pytest.mark.parametrize("full", [True, False])
def test_mul_u64_matches_oracle(ctx, devmem, m, full):
    n = 37 if m <= 256 else 5
    a, b = carry_stress(n, m, seed=31 * m + full)
    assert np.array_equal(gpu_mul(ctx, devmem, a, b, m, full), O.mul(a, b, m, full))


@pytest.mark.parametrize("m", [1, 3, 7, 9, 15, 255, 257, 511, 2047, 4095])
@pytest.mark.parametrize("full", [True, False])
def test_mul_u32_odd_sizes(ctx, devmem, m, full):
    n = 11
    a, b = carry_stress(n, m, seed=m, dtype=np.uint32)
    assert np.array_equal(gpu_mul(ctx, devmem, a, b, m, full, limb_bits=32), O.mul(a, b, m, full))


@pytest.mark.parametrize("m", [4, 128, 1024])
def test_mul_unaligned(ctx, devmem, m):
    a, b = carry_stress(6, m, seed=m + 1)
    for off in (1, 2):
        got = gpu_mul(ctx, devmem, a.view(np.uint32), b.view(np.uint32), 2 * m, True, limb_bits=32, offset=off)
        assert np.array_equal(got.view(np.uint64), O.mul(a, b, m, True))


@pytest.mark.parametrize("m", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096])
def test_mul_matches_reference_fixtures(ctx, devmem, m):
    g = golden("ref_sweep.npz")
    assert np.array_equal(gpu_mul(ctx, devmem, g["a"], g["b"], m, full=False, limb_bits=32), g[f"mul_{m}"])
    f = golden("ref_full.npz")
    ha, hb = f[f"ha_{m}"], f[f"hb_{m}"]
    n, h = ha.size // m, m // 2
    lo_a = np.ascontiguousarray(ha.reshape(n, m)[:, :h]).ravel()
    lo_b = np.ascontiguousarray(hb.reshape(n, m)[:, :h]).ravel()
    assert np.array_equal(gpu_mul(ctx, devmem, lo_a, lo_b, h, full=True, limb_bits=32), f[f"hmul_{m}"])
    w = golden("ref_worst.npz")
    assert np.array_equal(gpu_mul(ctx, devmem, w[f"wa_{m}"], w[f"wa_{m}"], m, False, 32), w[f"wmul_{m}"])


def test_mul_all_ones_full(ctx, devmem):
    for m in (1, 64, 128, 1024, 2048):
        a = np.full(3 * m, 0xFFFFFFFFFFFFFFFF, np.uint64)
        assert np.array_equal(gpu_mul(ctx, devmem, a, a, m, True), O.mul(a, a, m, True))


def test_mul_config_shape(ctx, devmem):
    import workloads

    a, b = workloads.mul_pairs(n=16384, m=128)
    got = gpu_mul(ctx, devmem, a, b, 128, True)
    assert np.array_equal(got, O.batch_u64("mul", a, b, 128, threads=16))
    # the u32-limb variant of the same workload is the same bytes
    got32 = gpu_mul(ctx, devmem, a.view(np.uint32)[: 256 * 64], b.view(np.uint32)[: 256 * 64], 256, True, 32)
    assert np.array_equal(got32.view(np.uint64), got[: 64 * 256])


@pytest.mark.parametrize("m", [255, 256, 300, 384, 447, 448, 500, 512, 1000, 1024, 1500, 2047, 2048])
@pytest.mark.parametrize("lo_min", [1, 2049])
def test_mul_lo_u64_classical_and_ntt(ctx, devmem, m, lo_min):
    """mi_mul_lo_u64 with the low-half crossover forced to the NTT (1) and to
    the classical kernel (2049): the same low limbs as the oracle."""
    old = ctx.get_tuning(midint.TUNE_LO_NTT_MIN)
    ctx.set_tuning(midint.TUNE_LO_NTT_MIN, 0, lo_min)
    try:
        a, b = carry_stress(7, m, seed=5 * m + lo_min)
        assert np.array_equal(gpu_mul(ctx, devmem, a, b, m, full=False), O.mul(a, b, m, False))
        ones = np.full(3 * m, 0xFFFFFFFFFFFFFFFF, np.uint64)
        assert np.array_equal(gpu_mul(ctx, devmem, ones, ones, m, full=False), O.mul(ones, ones, m, False))
    finally:
        ctx.set_tuning(midint.TUNE_LO_NTT_MIN, 0, old)


def test_lo_ntt_min_knob(ctx):
    old = ctx.get_tuning(midint.TUNE_LO_NTT_MIN)
    for bad in (0, 2050):
        with pytest.raises(midint.MidintError):
            ctx.set_tuning(midint.TUNE_LO_NTT_MIN, 0, bad)
    assert ctx.get_tuning(midint.TUNE_LO_NTT_MIN) == old
    ctx.set_tuning(midint.TUNE_LO_NTT_MIN, 0, 2049)
    assert ctx.get_tuning(midint.TUNE_LO_NTT_MIN) == 2049
    ctx.set_tuning(midint.TUNE_LO_NTT_MIN, 0, old)


def test_compat_gpuMultiply(lib):
    g = golden("ref_sweep.npz")
    for m in (16, 256, 1024, 2048, 4096):  # the u64 form of the last three takes the NTT low half
        r = np.zeros_like(g["a"])
        midint.gpuMultiply(midint.U32bits, m, g["a"].size // m, g["a"], g["b"], r)
        assert np.array_equal(r, g[f"mul_{m}"])
        a64, b64 = g["a"].view(np.uint64), g["b"].view(np.uint64)
        r64 = np.zeros_like(a64)
        midint.gpuMultiply(midint.U64bits, m // 2, a64.size // (m // 2), a64, b64, r64)
        assert np.array_equal(r64.view(np.uint32), g[f"mul_{m}"])


def test_host_mul_full(ctx):
    a, b = carry_stress(700, 128, seed=12)
    r = np.zeros(700 * 256, np.uint64)
    ctx.host_mul_full(a, b, r, 700, 128)
    assert np.array_equal(r, O.mul(a, b, 128, True))
