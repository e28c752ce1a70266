"""The oracle pinned against the reference's own answers (CPU only).

Golden fixtures were produced by the reference's CPU path (gmpAddMulOnce over
GMP, cuda/helper.h:146-170) on the reference's own inputs (ourMkRandom,
cuda/helper.h:99-114) for every size its benchmark sweeps
(cuda/main.cu:667-675, 693-703); the NTT vectors are the reference's own
known answers (futhark-clean/fft-mul.fut:355-406, cuda/main.cu:637-652).
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN, golden

SIZES = [16, 32, 64, 128, 256, 512, 1024, 2048, 4096]


@pytest.mark.parametrize("m", SIZES)
def test_add_matches_reference_sweep(m):
    g = golden("ref_sweep.npz")
    a, b = g["a"], g["b"]
    r, _ = O.add(a, b, m)                                   # u32 limbs
    assert np.array_equal(r, g[f"add_{m}"])
    if m % 2 == 0:                                          # same bytes as u64 limbs
        r64, _ = O.add(a.view(np.uint64), b.view(np.uint64), m // 2)
        assert np.array_equal(r64.view(np.uint32), g[f"add_{m}"])


@pytest.mark.parametrize("m", SIZES)
def test_mul_low_matches_reference_sweep(m):
    g = golden("ref_sweep.npz")
    a, b = g["a"], g["b"]
    assert np.array_equal(O.mul(a, b, m, full=False), g[f"mul_{m}"])
    r64 = O.mul(a.view(np.uint64), b.view(np.uint64), m // 2, full=False)
    assert np.array_equal(r64.view(np.uint32), g[f"mul_{m}"])


@pytest.mark.parametrize("m", SIZES)
def test_mul_full_matches_reference_on_half_filled_inputs(m):
    g = golden("ref_full.npz")
    ha, hb = g[f"ha_{m}"], g[f"hb_{m}"]
    n = ha.size // m
    h = m // 2
    # the top halves are zero, so the reference's m-word product is the full
    # product of the h-word low halves
    lo_a = ha.reshape(n, m)[:, :h].ravel()
    lo_b = hb.reshape(n, m)[:, :h].ravel()
    assert np.array_equal(O.mul(lo_a, lo_b, h, full=True), g[f"hmul_{m}"])


@pytest.mark.parametrize("m", SIZES)
def test_worst_case_carries(m):
    g = golden("ref_worst.npz")
    wa, wb = g[f"wa_{m}"], g[f"wb_{m}"]
    r, c = O.add(wa, wb, m)
    assert np.array_equal(r, g[f"wadd_{m}"]) and not r.any()
    assert c.all()
    assert np.array_equal(O.mul(wa, wa, m, full=False), g[f"wmul_{m}"])


def test_ntt_known_answers():
    v = json.load(open(os.path.join(GOLDEN, "ntt_vectors.json")))
    p, g, s = v["prime"]["p"], v["prime"]["g"], v["prime"]["two_adicity"]
    for f in v["forward"]:
        assert np.array_equal(O.ntt_forward(p, g, s, np.array(f["input"], np.uint64)),
                              np.array(f["output"], np.uint64))
    for c in v["conv"]:
        out = O.ntt_conv(p, g, s, np.array(c["a"], np.uint64), np.array(c["b"], np.uint64))
        assert np.array_equal(out, np.array(c["ref"], np.uint64))
        x = O.ntt_forward(p, g, s, np.array(c["a"], np.uint64))
        assert np.array_equal(O.ntt_inverse(p, g, s, x), np.array(c["a"], np.uint64))


@pytest.mark.parametrize("m", [1, 2, 3, 5, 8, 17, 64])
def test_oracle_vs_python_ints(m):
    rng = np.random.default_rng(m)
    a = rng.integers(0, 2**64, size=9 * m, dtype=np.uint64)
    b = rng.integers(0, 2**64, size=9 * m, dtype=np.uint64)
    a[:m] = np.uint64(2**64 - 1)
    b[:m] = 0
    b[0] = 1
    r, c = O.add(a, b, m)
    pr, pc = O.py_add(a, b, m)
    assert np.array_equal(r, pr) and np.array_equal(c, pc)
    assert np.array_equal(O.mul(a, b, m, True), O.py_mul(a, b, m, True))
    assert np.array_equal(O.mul(a, b, m, False), O.py_mul(a, b, m, False))
    a32, b32 = a.view(np.uint32), b.view(np.uint32)
    assert np.array_equal(O.mul(a32, b32, 2 * m, True).view(np.uint64), O.py_mul(a, b, m, True))
    assert np.array_equal(O.add6(a, b, m), O.from_ints([(6 * x + 10 * y) % (1 << (64 * m))
                                                        for x, y in zip(O.to_ints(a, m), O.to_ints(b, m))], m))
    mod = 1 << (64 * m)
    want = [((x * x + y) * (y * y + y) + x * y) % mod for x, y in zip(O.to_ints(a, m), O.to_ints(b, m))]
    assert np.array_equal(O.poly(a, b, m), O.from_ints(want, m))


def test_gmp_path_matches_restatement():
    if not O.gmp_available():
        pytest.skip("libgmp.so.10 not present")
    g = golden("ref_sweep.npz")
    for m in (16, 256, 4096):
        assert np.array_equal(O.gmp_batch(True, g["a"], g["b"], m, m, threads=2), g[f"add_{m}"])
        assert np.array_equal(O.gmp_batch(False, g["a"], g["b"], m, m, threads=2), g[f"mul_{m}"])
        full = O.gmp_batch(False, g["a"], g["b"], m, 2 * m, threads=3)
        assert np.array_equal(full, O.mul(g["a"], g["b"], m, full=True))


def test_multithreaded_batches():
    rng = np.random.default_rng(7)
    a = rng.integers(0, 2**64, size=37 * 24, dtype=np.uint64)
    b = rng.integers(0, 2**64, size=37 * 24, dtype=np.uint64)
    r, c = O.batch_u64("add", a, b, 24, threads=4)
    r1, c1 = O.add(a, b, 24)
    assert np.array_equal(r, r1) and np.array_equal(c, c1)
    assert np.array_equal(O.batch_u64("mul", a, b, 24, threads=5), O.mul(a, b, 24, True))


def test_reference_build_agrees_with_restatement():
    import build_ref

    path = build_ref.build()
    if path is None:
        pytest.skip("reference tree not present on this machine")
    import ctypes

    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    L.ref_gmp_add_mul.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, P, P, P]
    rng = np.random.default_rng(3)
    for m in (2, 64, 512):
        a = rng.integers(0, 2**32, size=5 * m, dtype=np.uint32)
        b = rng.integers(0, 2**32, size=5 * m, dtype=np.uint32)
        r = np.zeros_like(a)
        assert L.ref_gmp_add_mul(0, m, 5, a.ctypes.data_as(P), b.ctypes.data_as(P), r.ctypes.data_as(P)) == 0
        assert np.array_equal(r, O.mul(a, b, m, full=False))


def test_workload_generators_are_deterministic():
    import workloads as W

    # splitmix64 reference values for seed 0
    assert [hex(x) for x in W.splitmix64(0, 3)] == ["0xe220a8397b1dcdaf", "0x6e789e6aa1b965f4", "0x6c45d188009454f"]
    a, b = W.add_pairs(n=16, m=4)
    assert (a.reshape(16, 4)[::8] == np.uint64(2**64 - 1)).all()
    assert (b.reshape(16, 4)[::8, 0] == 1).all() and not b.reshape(16, 4)[::8, 1:].any()
    a2, _ = W.add_pairs(n=16, m=4)
    assert np.array_equal(a, a2)


FORMATS = [(order, size, endian) for order in (-1, 1) for size in (1, 2, 4, 8) for endian in (-1, 0, 1)]


@pytest.mark.parametrize("order,size,endian", FORMATS)
def test_word_formats_match_gmp(order, size, endian):
    """The import/export restatement against GMP's own mpz_import/mpz_export."""
    if not O.gmp_available():
        pytest.skip("libgmp.so.10 not present")
    rng = np.random.default_rng(size * 7 + order + endian)
    limbs = 5
    for words in (1, 3, 40 // size, 40 // size + 3):
        n = 4
        x = rng.integers(0, 2**64, size=n * limbs, dtype=np.uint64)
        x[limbs:2 * limbs] = 0                             # a zero value
        x[2 * limbs + 2:3 * limbs] = 0                     # a short value
        field, counts = O.export_words(x, n, limbs, words, size, order, endian)
        back = O.import_words(field, n, words, size, order, endian, limbs)
        for i in range(n):
            xi = x[i * limbs:(i + 1) * limbs]
            f, cnt = O.gmp_export(xi, words, size, order, endian)
            assert cnt == counts[i]
            if cnt <= words:
                assert np.array_equal(f, field[i * words * size:(i + 1) * words * size])
                assert np.array_equal(back[i * limbs:(i + 1) * limbs], xi)
            g, _ = O.gmp_import(field[i * words * size:(i + 1) * words * size], words, size, order, endian, limbs)
            assert np.array_equal(g, back[i * limbs:(i + 1) * limbs])


def test_reference_word_format_is_u32_least_first():
    # cuda/helper.h:116-170 imports and exports order -1, 4-byte native words:
    # the same bytes as the library's u64 limbs
    rng = np.random.default_rng(1)
    x = rng.integers(0, 2**64, size=3 * 4, dtype=np.uint64)
    field, _ = O.export_words(x, 3, 4, 8, 4, -1, 0)
    assert np.array_equal(field.view(np.uint64), x)
