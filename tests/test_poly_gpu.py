"""GPU fused composite ((a^2 + b)(b^2 + b) + ab) mod 2^(64m) vs the oracle.

The composite is the reference's polyKerQ (cuda/ker-classic-mul.cu.h:500-575):
every intermediate is reduced mod 2^(64m), as its wrapper of m-limb products
and sums does.
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


@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 8, 16, 17, 32, 33, 64, 100, 128, 256, 257, 512, 1024, 1500, 2048])
def test_poly_matches_oracle(ctx, devmem, m):
    n = 41 if m <= 128 else 6
    a, b = carry_stress(n, m, seed=7 * m + 3)
    assert np.array_equal(gpu_poly(ctx, devmem, a, b, m), O.poly(a, b, m))


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


def test_poly_unaligned_rows(ctx, devmem):
    m = 64
    a, b = carry_stress(5, m, seed=99)
    assert np.array_equal(gpu_poly(ctx, devmem, a, b, m, offset=1), O.poly(a, b, m))


def test_poly_rejects_bad_arguments(ctx):
    with pytest.raises(midint.MidintError):
        ctx.poly(0, 16, 32, 1, 4)
    with pytest.raises(midint.MidintError):
        ctx.poly(16, 16, 16 + 8, 1, 2049)
    ctx.poly(16, 16, 4096, 0, 4)  # empty batch: nothing launched
