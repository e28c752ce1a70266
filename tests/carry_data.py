"""Seeded operands that stress carry propagation.

Each limb pair is drawn as one of: generate (both near all-ones, sum
overflows), propagate (a + b is exactly all ones), kill (both small) or
uniform.  Long propagate runs make carries cross thread, warp and block
boundaries of the GPU kernels; rows of all-ones + 1 and ~x + x + 1 give
carries through the whole integer.
"""
from __future__ import annotations

import numpy as np

MAX64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def carry_stress(n: int, m: int, seed: int, dtype=np.uint64):
    rng = np.random.default_rng(seed)
    bits = np.dtype(dtype).itemsize * 8
    top = (1 << bits) - 1
    a = rng.integers(0, top, size=(n, m), dtype=np.uint64, endpoint=True).astype(dtype)
    b = rng.integers(0, top, size=(n, m), dtype=np.uint64, endpoint=True).astype(dtype)
    kind = rng.choice(4, size=(n, m), p=[0.1, 0.6, 0.1, 0.2])
    allones = dtype(top)
    # propagate: b = ~a
    prop = kind == 1
    b[prop] = allones - a[prop]
    # generate: both in the top half
    gen = kind == 0
    a[gen] |= dtype(1 << (bits - 1))
    b[gen] |= dtype(1 << (bits - 1))
    # kill: both small
    kill = kind == 2
    a[kill] >>= dtype(bits // 2)
    b[kill] >>= dtype(bits // 2)
    # whole-integer chains on a few rows
    if n >= 3:
        a[0, :] = allones
        b[0, :] = 0
        b[0, 0] = 1
        a[1, :] = rng.integers(0, top, size=m, dtype=np.uint64, endpoint=True).astype(dtype)
        b[1, :] = allones - a[1, :]
        b[1, 0] += dtype(1) if a[1, 0] != 0 else dtype(0)
        a[2, :] = allones
        b[2, :] = allones
    return a.ravel(), b.ravel()
