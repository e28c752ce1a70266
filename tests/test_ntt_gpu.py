"""GPU NTT: the transform against the reference's known answers, and exact
NTT multiplication against the oracle, bit-exact, through the C ABI."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest
import torch

import midint
import oracle as O
from carry_data import carry_stress
from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu

FFT_PRIME64 = (29 * 2**57 + 1, 21, 57)   # cuda/ker-fft-mul.cu.h:44-57


def test_transform_matches_reference_known_answers(lib):
    v = json.load(open(os.path.join(GOLDEN, "ntt_vectors.json")))
    p, g, s = v["prime"]["p"], v["prime"]["g"], v["prime"]["two_adicity"]
    for f in v["forward"]:
        got = midint.ntt_raw(p, g, s, np.array(f["input"], np.uint64))
        assert np.array_equal(got, np.array(f["output"], np.uint64))
    for c in v["conv"]:
        got = midint.ntt_raw(p, g, s, np.array(c["a"], np.uint64), np.array(c["b"], np.uint64))
        assert np.array_equal(got, np.array(c["ref"], np.uint64))


@pytest.mark.parametrize("length", [8, 16, 64, 256, 512, 1024, 2048])
def test_transform_on_reference_prime64_matches_oracle(lib, length):
    p, g, s = FFT_PRIME64
    rng = np.random.default_rng(length)
    a = rng.integers(0, p, size=length, dtype=np.uint64)
    b = rng.integers(0, p, size=length, dtype=np.uint64)
    assert np.array_equal(midint.ntt_raw(p, g, s, a), O.ntt_forward(p, g, s, a))
    assert np.array_equal(midint.ntt_raw(p, g, s, a, b), O.ntt_conv(p, g, s, a, b))


def test_transform_generic_field_matches_oracle(lib):
    p, g, s = 3221225473, 13, 30            # FftPrime32: p != 1 mod 2^32
    rng = np.random.default_rng(5)
    for length in (8, 128, 2048):
        a = rng.integers(0, p, size=length, dtype=np.uint64)
        b = rng.integers(0, p, size=length, dtype=np.uint64)
        assert np.array_equal(midint.ntt_raw(p, g, s, a, b), O.ntt_conv(p, g, s, a, b))


def _stream():
    return torch.cuda.current_stream().cuda_stream


def gpu_mul_ntt(ctx, devmem, a, b, m, via="ntt"):
    n = a.size // m
    ba, pa = devmem.put(a)
    bb, pb = devmem.put(b)
    br, pr = devmem.empty_words(4 * a.size)
    (ctx.mul_ntt if via == "ntt" else ctx.mul)(pa, pb, pr, n, m, stream=_stream())
    torch.cuda.synchronize()
    assert (br[4 * a.size:].cpu().numpy() == -1).all(), "result written past the batch"
    return devmem.get(br, 4 * a.size)


NTT_SIZES = [1, 2, 3, 63, 64, 65, 100, 127, 128, 129, 255, 256, 257, 500, 511, 512, 513, 1000, 1023, 1024, 1025,
             1500, 2047, 2048]


@pytest.mark.parametrize("m", NTT_SIZES)
def test_mul_ntt_matches_oracle(ctx, devmem, m):
    n = 9 if m <= 256 else 4
    a, b = carry_stress(n, m, seed=77 * m)
    assert np.array_equal(gpu_mul_ntt(ctx, devmem, a, b, m), O.mul(a, b, m, True))


# sizes whose 40-bit digits fit the transform length (three primes): 80 and
# 320 limbs fill 256 and 1024 points exactly, 525 limbs is the largest
# shorter operand the three primes keep exact (840 digits), 526 the first
# that falls back to 48-bit digits on four
D40_SIZES = [10, 40, 76, 80, 150, 160, 300, 320, 321, 400, 520, 525, 526]


@pytest.mark.parametrize("m", D40_SIZES)
def test_mul_ntt_40bit_digits_match_oracle(ctx, devmem, m):
    a, b = carry_stress(6, m, seed=31 * m + 1)
    assert np.array_equal(gpu_mul_ntt(ctx, devmem, a, b, m), O.mul(a, b, m, True))


@pytest.mark.parametrize("m", [64, 80, 96, 256, 320, 384, 525, 526, 1024, 1536, 2048])
def test_mul_ntt_maximal_coefficients(ctx, devmem, m):
    # all-ones operands give the largest convolution coefficients (~m * 2^128
    # with 64-bit digits; 96, 384 and 1536 limbs fill their transform length
    # exactly with 48-bit digits on four primes, coefficients ~(4m/3) * 2^96;
    # 80 and 320 limbs fill it with 40-bit digits on three, and 525 limbs
    # reach the three primes' bound, 840 (2^40 - 1)^2)
    a = np.full(3 * m, 0xFFFFFFFFFFFFFFFF, np.uint64)
    b = a.copy()
    b[m:2 * m] = 1
    assert np.array_equal(gpu_mul_ntt(ctx, devmem, a, b, m), O.mul(a, b, m, True))


@pytest.mark.parametrize("m", [1, 64, 95, 96, 97, 100, 159, 160, 255, 256, 700, 1024, 2048])
def test_mul_dispatch_matches_oracle(ctx, devmem, m):
    # either side of the tuned classical/NTT crossover of mi_mul_u64
    a, b = carry_stress(5, m, seed=m + 3)
    assert np.array_equal(gpu_mul_ntt(ctx, devmem, a, b, m, via="dispatch"), O.mul(a, b, m, True))


def test_mul_ntt_config_shape(ctx, devmem):
    import workloads

    a, b = workloads.ntt_pairs(n=1024, m=1024)
    got = gpu_mul_ntt(ctx, devmem, a, b, 1024)
    assert np.array_equal(got, O.batch_u64("mul", a, b, 1024, threads=16))


def test_mul_ntt_matches_classical_on_reference_fixtures(ctx, devmem):
    f = golden("ref_full.npz")
    for m in (256, 1024, 2048, 4096):            # u32 words; the products fit m words
        ha, hb = f[f"ha_{m}"], f[f"hb_{m}"]
        n, h = ha.size // m, m // 2
        lo_a = np.ascontiguousarray(ha.reshape(n, m)[:, :h]).ravel().view(np.uint64)
        lo_b = np.ascontiguousarray(hb.reshape(n, m)[:, :h]).ravel().view(np.uint64)
        got = gpu_mul_ntt(ctx, devmem, lo_a, lo_b, h // 2)
        assert np.array_equal(got.view(np.uint32), f[f"hmul_{m}"])


def test_compat_gpuMulFFT(lib):
    g = golden("ref_sweep.npz")
    for m32 in (64, 256, 2048, 4096):
        M = 2 * m32                                # u16 digits
        a16 = g["a"].view(np.uint16)
        b16 = g["b"].view(np.uint16)
        n = a16.size // M
        rs = np.zeros(n * M, np.uint32)
        midint.gpuMulFFT(midint.FftPrime32, M, n, a16, b16, rs)
        # the low M digits of every product packed at digit offset i*M, i.e.
        # the reference's gmpMultiply<m32> words; the second half is untouched
        got = rs.view(np.uint16)[: n * M].view(np.uint32)
        assert np.array_equal(got, g[f"mul_{m32}"])
        assert not rs[n * M // 2:].any()


# --- the production transform (ntt32.cuh) on its own ---------------------------

def _order_2s(p: int, g: int) -> tuple[int, int]:
    """(g', s): g' = g^((p-1)/2^s) of order 2^s, s the 2-adicity of p - 1, so
    the oracle's root for length L, g'^(2^s / L), is g^((p-1)/L)."""
    s = ((p - 1) & -(p - 1)).bit_length() - 1
    return pow(g, (p - 1) >> s, p), s


@pytest.mark.parametrize("q", range(5))
@pytest.mark.parametrize("length", [256, 512, 1024, 2048, 4096])
def test_production_transform_matches_oracle(ctx, q, length):
    p, g = midint.ntt32_prime(q)
    g2, s = _order_2s(p, g)
    rng = np.random.default_rng(1000 * q + length)
    a = rng.integers(0, p, size=length, dtype=np.uint64)
    b = rng.integers(0, p, size=length, dtype=np.uint64)
    fwd = midint.ntt32_raw(ctx, q, a.astype(np.uint32))
    assert np.array_equal(fwd.astype(np.uint64), O.ntt_forward(p, g2, s, a))
    conv = midint.ntt32_raw(ctx, q, a.astype(np.uint32), b.astype(np.uint32))
    assert np.array_equal(conv.astype(np.uint64), O.ntt_conv(p, g2, s, a, b))


@pytest.mark.parametrize("q", [0, 4])
@pytest.mark.parametrize("length", [256, 4096])
def test_production_transform_edge_residues(ctx, q, length):
    p, g = midint.ntt32_prime(q)
    g2, s = _order_2s(p, g)
    top = np.full(length, p - 1, np.uint64)              # the largest residues
    delta = np.zeros(length, np.uint64)
    delta[0] = 1
    assert (midint.ntt32_raw(ctx, q, delta.astype(np.uint32)) == 1).all()   # spectrum of a unit impulse
    assert np.array_equal(midint.ntt32_raw(ctx, q, top.astype(np.uint32)).astype(np.uint64),
                          O.ntt_forward(p, g2, s, top))
    assert np.array_equal(midint.ntt32_raw(ctx, q, top.astype(np.uint32), top.astype(np.uint32)).astype(np.uint64),
                          O.ntt_conv(p, g2, s, top, top))
    # inputs at or above p are reduced mod p first
    big = np.full(length, 0xFFFFFFFF, np.uint64)
    assert np.array_equal(midint.ntt32_raw(ctx, q, big.astype(np.uint32)).astype(np.uint64),
                          O.ntt_forward(p, g2, s, big % p))


def test_mul_ntt_rejects_misaligned_buffers(ctx, devmem):
    # the transform kernels read 8-byte words: 4-byte aligned rows are refused
    # on the host (the size-dispatched entry points take the classical kernel)
    a, b = carry_stress(2, 300, seed=5)
    ba, pa = devmem.put(a, 1)
    bb, pb = devmem.put(b, 1)
    br, pr = devmem.empty_words(4 * a.size, 1)
    with pytest.raises(midint.MidintError) as e:
        ctx.mul_ntt(pa, pb, pr, 2, 300, stream=_stream())
    assert e.value.status == midint.MI_EINVAL


@pytest.mark.parametrize("m", [200, 400, 2048])
def test_size_dispatch_on_misaligned_rows_matches_oracle(ctx, devmem, m):
    a, b = carry_stress(3, m, seed=m + 9)
    ba, pa = devmem.put(a, 1)
    bb, pb = devmem.put(b, 1)
    br, pr = devmem.empty_words(4 * a.size, 1)
    ctx.mul(pa, pb, pr, 3, m, stream=_stream())
    torch.cuda.synchronize()
    assert np.array_equal(devmem.get(br, 4 * a.size, 1), O.mul(a, b, m, True))
    br2, pr2 = devmem.empty_words(2 * a.size, 1)
    ctx.mul_lo(pa, pb, pr2, 3, m, stream=_stream())
    torch.cuda.synchronize()
    assert np.array_equal(devmem.get(br2, 2 * a.size, 1), O.mul(a, b, m, False))
