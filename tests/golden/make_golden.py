"""Generates the committed golden fixtures from the reference's own CPU path.

Run in a checkout that has the reference tree (it compiles oracle/_ref with
oracle/build_ref.py); the fixtures it writes are what tests/ use everywhere
else.  Inputs come from the reference's own generator ourMkRandom
(cuda/helper.h:99-114) after srand(1) -- glibc's default seed, i.e. what
cuda/main.cu's mkRandArrays<32,32> produces (cuda/main.cu:18-33) -- and
outputs from its gmpAdd / gmpMultiply loops over gmpAddMulOnce
(cuda/main.cu:165-175, 358-368; cuda/helper.h:146-170), for every size the
reference's runAdditions / runNaiveMuls sweep (cuda/main.cu:667-675, 693-703).

  ref_sweep.npz : a, b (4096 u32 words each) and, per size m in u32 words,
                  add_<m> = (a + b) mod 2^(32m), mul_<m> = a*b mod 2^(32m)
  ref_full.npz  : half-filled inputs (ourMkRandom<m, m/2>) so the product fits
                  in m words: ha_<m>, hb_<m>, hmul_<m> = full product
  ref_worst.npz : all-ones + 1 carry chains per size (sum 0, carry out 1)
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402

WORDS = 4096
SIZES = [16, 32, 64, 128, 256, 512, 1024, 2048, 4096]


def main() -> None:
    path = build_ref.build()
    if path is None:
        raise SystemExit("reference tree not present: cannot generate fixtures")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    L.ref_gmp_add_mul.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, P, P, P]
    L.ref_mk_random.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, P]
    L.ref_srand.argtypes = [ctypes.c_uint]

    def p(x):
        return x.ctypes.data_as(P)

    def run(is_add, m, a, b):
        n = a.size // m
        r = np.zeros(a.size, np.uint32)
        assert L.ref_gmp_add_mul(1 if is_add else 0, m, n, p(a), p(b), p(r)) == 0
        return r

    L.ref_srand(1)
    a = np.zeros(WORDS, np.uint32)
    b = np.zeros(WORDS, np.uint32)
    assert L.ref_mk_random(32, 32, WORDS // 32, p(a)) == 0
    assert L.ref_mk_random(32, 32, WORDS // 32, p(b)) == 0
    sweep = {"a": a, "b": b}
    for m in SIZES:
        sweep[f"add_{m}"] = run(True, m, a, b)
        sweep[f"mul_{m}"] = run(False, m, a, b)
    np.savez_compressed(os.path.join(HERE, "ref_sweep.npz"), **sweep)

    full = {}
    for m in SIZES:
        ha = np.zeros(WORDS, np.uint32)
        hb = np.zeros(WORDS, np.uint32)
        assert L.ref_mk_random(m, m // 2, WORDS // m, p(ha)) == 0
        assert L.ref_mk_random(m, m // 2, WORDS // m, p(hb)) == 0
        full[f"ha_{m}"], full[f"hb_{m}"] = ha, hb
        full[f"hmul_{m}"] = run(False, m, ha, hb)
    np.savez_compressed(os.path.join(HERE, "ref_full.npz"), **full)

    worst = {}
    for m in SIZES:
        n = max(1, 256 // m)
        wa = np.full(n * m, 0xFFFFFFFF, np.uint32)
        wb = np.zeros(n * m, np.uint32)
        wb[::m] = 1
        worst[f"wa_{m}"], worst[f"wb_{m}"] = wa, wb
        worst[f"wadd_{m}"] = run(True, m, wa, wb)
        worst[f"wmul_{m}"] = run(False, m, wa, wa)
    np.savez_compressed(os.path.join(HERE, "ref_worst.npz"), **worst)
    print("wrote ref_sweep.npz ref_full.npz ref_worst.npz")


if __name__ == "__main__":
    main()
