"""GPU fused composite ((a^2 + b)(b^2 + b) + ab) mod 2^(64m) vs the oracle.

The composite is the reference's polyKerQ (cuda/ker-classic-mul.cu.h:500-575)
and, on transforms, its polyFttKer (cuda/ker-fft-mul.cu.h:456-509): every
intermediate is reduced mod 2^(64m), as its wrapper of m-limb products and
sums does.  Both forms (classical low halves, and low halves on exact
number-theoretic transforms) are run at every size by setting the crossover
knob, so each is checked whatever the tuned crossover is.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import midint
import oracle as O
from carry_data import carry_stress

pytestmark = pytest.mark.gpu


def gpu_poly(ctx, devmem, a, b, m, offset=0):
    n = a.size // m
    words = a.view(np.uint32).size
    ba, pa = devmem.put(a, offset)
    bb, pb = devmem.put(b, offset)
    br, pr = devmem.empty_words(words, offset)
    ctx.poly(pa, pb, pr, n, m, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert (br[offset + words:].cpu().numpy() == -1).all(), "result written past the batch"
    return devmem.get(br, words, offset)


@pytest.fixture(params=["classical", "ntt"])
def form(request, ctx):
    """Runs the test with mi_poly_u64 forced to one form."""
    old = ctx.get_tuning(midint.TUNE_POLY_NTT_MIN)
    ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, 2049 if request.param == "classical" else 1)
    yield request.param
    ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, old)


@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 8, 16, 17, 32, 33, 64, 96, 100, 128, 129, 200, 256, 257, 320, 384,
                               500, 512, 700, 1024, 1500, 1536, 2048])
def test_poly_matches_oracle(ctx, devmem, form, m):
    n = 41 if m <= 128 else 6
    a, b = carry_stress(n, m, seed=7 * m + 3)
    assert np.array_equal(gpu_poly(ctx, devmem, a, b, m), O.poly(a, b, m))


@pytest.mark.parametrize("m", [3, 96, 384, 1536, 2048])
def test_poly_all_ones(ctx, devmem, form, m):
    # all-ones operands give the largest transform coefficients (96, 384 and
    # 1536 limbs fill their length exactly with 48-bit digits on four primes)
    n = 4
    a = np.full(n * m, 0xFFFFFFFFFFFFFFFF, np.uint64)
    b = a.copy()
    b[m:2 * m] = 1                       # one pair with b = 1 .. 1
    b[3 * m:] = 0                        # one pair with b = 0
    assert np.array_equal(gpu_poly(ctx, devmem, a, b, m), O.poly(a, b, m))


def test_poly_ntt_config_shape(ctx, devmem):
    """The 2048-limb composite on a batch that fills the GPU several times,
    checked against the oracle on every instance."""
    import workloads

    old = ctx.get_tuning(midint.TUNE_POLY_NTT_MIN)
    ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, 1)
    try:
        a, b = workloads.mul_pairs(n=400, m=2048, seed=workloads.SEED_BASE + 11)
        assert np.array_equal(gpu_poly(ctx, devmem, a, b, 2048), O.poly(a, b, 2048))
    finally:
        ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, old)


def test_poly_small_vs_python_ints(ctx, devmem):
    m = 3
    rng = np.random.default_rng(11)
    a = rng.integers(0, 2**64, size=50 * m, dtype=np.uint64)
    b = rng.integers(0, 2**64, size=50 * m, dtype=np.uint64)
    a[:m] = np.uint64(2**64 - 1)
    b[m:2 * m] = np.uint64(2**64 - 1)
    mod = 1 << (64 * m)
    want = [((x * x + y) * (y * y + y) + x * y) % mod for x, y in zip(O.to_ints(a, m), O.to_ints(b, m))]
    assert np.array_equal(gpu_poly(ctx, devmem, a, b, m), O.from_ints(want, m))


@pytest.mark.parametrize("m", [64, 400])
def test_poly_unaligned_rows(ctx, devmem, form, m):
    a, b = carry_stress(5, m, seed=99 + m)
    assert np.array_equal(gpu_poly(ctx, devmem, a, b, m, offset=1), O.poly(a, b, m))


def test_poly_crossover_knob_bounds(ctx):
    old = ctx.get_tuning(midint.TUNE_POLY_NTT_MIN)
    for bad in (0, 2050):
        with pytest.raises(midint.MidintError):
            ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, bad)
    assert ctx.get_tuning(midint.TUNE_POLY_NTT_MIN) == old


def test_poly_rejects_bad_arguments(ctx):
    with pytest.raises(midint.MidintError):
        ctx.poly(0, 16, 32, 1, 4)
    with pytest.raises(midint.MidintError):
        ctx.poly(16, 16, 16 + 8, 1, 2049)
    ctx.poly(16, 16, 4096, 0, 4)  # empty batch: nothing launched
