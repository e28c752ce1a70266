"""Seeded synthetic batches with the shapes of the benchmark workloads.

All limbs come from splitmix64 streams (seed -> 64-bit words), so every run,
here and on any other machine, sees the same integers.  Workloads:

* plain addition: 65536 pairs of 4096-bit integers (64 u64 limbs), uniform,
  with every 8th pair a worst-case carry chain (A all ones, B = 1);
* classical multiplication: 16384 pairs of 8192-bit integers (128 u64 limbs ->
  256-limb product), uniform; the u32 variant is the same bytes as 256 u32 limbs;
* NTT multiplication: 1024 pairs of 65536-bit integers (1024 u64 limbs),
  uniform, with every 16th pair all ones (maximal coefficients);
* ragged batch: 200000 operations, 40 % additions / 60 % multiplications,
  each operand's bit length drawn independently log-uniform in [256, 65536]
  and rounded up to whole u64 limbs (4 ... 1024 limbs), uniform limbs.

The reference's own generator (ourMkRandom, cuda/helper.h:99-114) builds
words from glibc rand() and never sets the low bit, so it almost never
produces long carry chains; the worst-case pairs here are added on purpose.
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 0x5EED0000
_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, start: int = 0) -> np.ndarray:
    """Outputs start .. start+count-1 of splitmix64 started at `seed`."""
    with np.errstate(over="ignore"):
        x = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + _GOLD * np.arange(start + 1, start + count + 1, dtype=np.uint64)
        z = (x ^ (x >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(n: int, m: int, seed: int, first: int = 0) -> np.ndarray:
    """Instances first .. first+n-1 (m limbs each) of one seeded stream."""
    return splitmix64(seed, n * m, first * m)


def add_pairs(n: int = 65536, m: int = 64, seed: int = SEED_BASE + 0, worst_every: int = 8, first: int = 0):
    """Addition workload: (a, b) flat u64 arrays of n*m limbs (instances
    first .. first+n-1 of the seeded batch)."""
    a = uniform(n, m, seed, first)
    b = uniform(n, m, seed ^ 0xB0B0B0B0, first)
    if worst_every:
        rows = np.arange((-first) % worst_every, n, worst_every)
        a2, b2 = a.reshape(n, m), b.reshape(n, m)
        a2[rows, :] = np.uint64(0xFFFFFFFFFFFFFFFF)
        b2[rows, :] = 0
        b2[rows, 0] = 1
    return a, b


def mul_pairs(n: int = 16384, m: int = 128, seed: int = SEED_BASE + 1, first: int = 0):
    """Classical-multiplication workload: uniform (a, b) of n*m u64 limbs
    (instances first .. first+n-1 of the seeded batch)."""
    return uniform(n, m, seed, first), uniform(n, m, seed ^ 0xB0B0B0B0, first)


def ntt_pairs(n: int = 1024, m: int = 1024, seed: int = SEED_BASE + 2, ones_every: int = 16, first: int = 0):
    """NTT-multiplication workload: uniform, every 16th pair all ones
    (instances first .. first+n-1 of the seeded batch)."""
    a = uniform(n, m, seed, first)
    b = uniform(n, m, seed ^ 0xB0B0B0B0, first)
    if ones_every:
        rows = np.arange((-first) % ones_every, n, ones_every)
        a.reshape(n, m)[rows, :] = np.uint64(0xFFFFFFFFFFFFFFFF)
        b.reshape(n, m)[rows, :] = np.uint64(0xFFFFFFFFFFFFFFFF)
    return a, b


def ragged_ops(n_ops: int = 200000, seed: int = SEED_BASE + 3, add_frac: float = 0.4,
               min_bits: int = 256, max_bits: int = 65536):
    """Ragged workload: (ops, pool_in, out_limbs).

    ops: structured array of mi_op records (midint.OP_DTYPE layout); operands
    packed a0 b0 a1 b1 ... in pool_in (u64); results packed in op order in an
    output pool of out_limbs limbs (max(la, lb) per add, la + lb per mul)."""
    rng = np.random.default_rng(seed)
    kind = (rng.random(n_ops) >= add_frac).astype(np.uint32)  # 0 add, 1 mul
    lo, hi = np.log(min_bits), np.log(max_bits)
    la = np.ceil(np.exp(rng.uniform(lo, hi, n_ops)) / 64).astype(np.uint32)
    lb = np.ceil(np.exp(rng.uniform(lo, hi, n_ops)) / 64).astype(np.uint32)
    return pack_ops(kind, la, lb, seed)


def pack_ops(kind: np.ndarray, la: np.ndarray, lb: np.ndarray, seed: int):
    """mi_op records for the given kinds and lengths, with seeded operands."""
    n = kind.size
    dt = np.dtype([("kind", "<u4"), ("la", "<u4"), ("lb", "<u4"), ("flags", "<u4"),
                   ("a_off", "<u8"), ("b_off", "<u8"), ("r_off", "<u8")])
    ops = np.zeros(n, dt)
    ops["kind"], ops["la"], ops["lb"] = kind, la, lb
    pair = la.astype(np.uint64) + lb.astype(np.uint64)
    starts = np.concatenate([[0], np.cumsum(pair)[:-1]]).astype(np.uint64)
    ops["a_off"] = starts
    ops["b_off"] = starts + la.astype(np.uint64)
    rlen = np.where(kind == 0, np.maximum(la, lb), la + lb).astype(np.uint64)
    ops["r_off"] = np.concatenate([[0], np.cumsum(rlen)[:-1]]).astype(np.uint64)
    pool = splitmix64(seed ^ 0x7A99ED, int(pair.sum()))
    return ops, pool, int(rlen.sum())
