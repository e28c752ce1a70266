"""THE ORACLE (Python side).  Test infrastructure only.

Wraps oracle/orc.c (the CPU restatement of the reference's add / classical
mul / NTT algorithms and of its GMP CPU path, see the header of orc.c for the
file:line each function follows) with numpy-facing functions, plus pure-Python
`int` cross-oracles for small cases.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this module; the library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "orc.c")
LIB = os.path.join(HERE, "liborc.so")

_lib = None


def build(force: bool = False) -> str:
    """Compiles orc.c into liborc.so with gcc (a second or two)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["gcc", "-O2", "-std=gnu11", "-shared", "-fPIC", "-pthread", SRC, "-o", LIB, "-ldl"]
        subprocess.run(cmd, check=True)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        u64, u32, i32 = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
        L.orc_add_u64.argtypes = [u64, u32, P, P, P, P]
        L.orc_add_u32.argtypes = [u64, u32, P, P, P, P]
        L.orc_add6_u64.argtypes = [u64, u32, P, P, P]
        L.orc_poly_u64.argtypes = [u64, u32, P, P, P]
        L.orc_mul_u64.argtypes = [u64, u32, P, P, P, i32]
        L.orc_mul_u32.argtypes = [u64, u32, P, P, P, i32]
        for f in ("orc_zmod_mul", "orc_zmod_add", "orc_zmod_sub", "orc_zmod_pow"):
            getattr(L, f).argtypes = [u64, u64, u64]
            getattr(L, f).restype = u64
        L.orc_zmod_inv.argtypes = [u64, u64]
        L.orc_zmod_inv.restype = u64
        L.orc_ntt_omega.argtypes = [u64, u64, u32, u32]
        L.orc_ntt_omega.restype = u64
        L.orc_ntt_forward.argtypes = [u64, u64, u32, u32, P, P]
        L.orc_ntt_inverse.argtypes = [u64, u64, u32, u32, P, P]
        L.orc_ntt_conv.argtypes = [u64, u64, u32, u32, P, P, P]
        L.orc_gmp_available.restype = i32
        L.orc_gmp_batch.argtypes = [i32, u64, u32, P, P, P, u32, i32]
        L.orc_gmp_batch.restype = i32
        L.orc_batch_u64.argtypes = [i32, u64, u32, P, P, P, P, i32]
        L.orc_gmp_import.argtypes = [P, u32, i32, u32, i32, P, u32]
        L.orc_gmp_import.restype = i32
        L.orc_gmp_export.argtypes = [P, u32, i32, u32, i32, P, u32]
        L.orc_gmp_export.restype = i32
        _lib = L
    return _lib


def _p(x: np.ndarray | None):
    return None if x is None else x.ctypes.data_as(ctypes.c_void_p)


def _c(x: np.ndarray, dtype) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=dtype)


# --- addition ---------------------------------------------------------------

def add(a: np.ndarray, b: np.ndarray, m: int, with_carry: bool = True):
    """(a + b) mod 2^(bits*m) per instance, and the carry-out bits.

    a, b: flat uint64 or uint32 arrays of n*m limbs."""
    dt = a.dtype
    a, b = _c(a, dt), _c(b, dt)
    n = a.size // m
    r = np.empty_like(a)
    c = np.zeros(n, np.uint8) if with_carry else None
    f = lib().orc_add_u64 if dt == np.uint64 else lib().orc_add_u32
    f(n, m, _p(a), _p(b), _p(r), _p(c))
    return (r, c) if with_carry else r


def add6(a: np.ndarray, b: np.ndarray, m: int) -> np.ndarray:
    """6a + 10b mod 2^(64m) per instance (u64 limbs)."""
    a, b = _c(a, np.uint64), _c(b, np.uint64)
    r = np.empty_like(a)
    lib().orc_add6_u64(a.size // m, m, _p(a), _p(b), _p(r))
    return r


def poly(a: np.ndarray, b: np.ndarray, m: int) -> np.ndarray:
    """((a^2 + b)(b^2 + b) + ab) mod 2^(64m) per instance (u64 limbs)."""
    a, b = _c(a, np.uint64), _c(b, np.uint64)
    r = np.empty_like(a)
    lib().orc_poly_u64(a.size // m, m, _p(a), _p(b), _p(r))
    return r


# --- classical multiplication -----------------------------------------------

def mul(a: np.ndarray, b: np.ndarray, m: int, full: bool = True) -> np.ndarray:
    """a*b per instance: 2m limbs (full) or the low m limbs."""
    dt = a.dtype
    a, b = _c(a, dt), _c(b, dt)
    n = a.size // m
    r = np.empty(n * m * (2 if full else 1), dt)
    f = lib().orc_mul_u64 if dt == np.uint64 else lib().orc_mul_u32
    f(n, m, _p(a), _p(b), _p(r), 1 if full else 0)
    return r


# --- NTT primitives of the reference ------------------------------------------

def ntt_forward(p: int, g: int, two_adicity: int, x: np.ndarray) -> np.ndarray:
    x = _c(x, np.uint64)
    out = np.empty_like(x)
    lib().orc_ntt_forward(p, g, two_adicity, x.size, _p(x), _p(out))
    return out


def ntt_inverse(p: int, g: int, two_adicity: int, x: np.ndarray) -> np.ndarray:
    x = _c(x, np.uint64)
    out = np.empty_like(x)
    lib().orc_ntt_inverse(p, g, two_adicity, x.size, _p(x), _p(out))
    return out


def ntt_conv(p: int, g: int, two_adicity: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a, b = _c(a, np.uint64), _c(b, np.uint64)
    out = np.empty_like(a)
    lib().orc_ntt_conv(p, g, two_adicity, a.size, _p(a), _p(b), _p(out))
    return out


# --- GMP path (the reference's CPU path) ---------------------------------------

def gmp_available() -> bool:
    return bool(lib().orc_gmp_available())


def gmp_batch(is_add: bool, a32: np.ndarray, b32: np.ndarray, m32: int, out_words: int,
              threads: int = 1) -> np.ndarray:
    """gmpAddMulOnce over a batch of m32-word u32 instances (cuda/helper.h:146-170)."""
    a32, b32 = _c(a32, np.uint32), _c(b32, np.uint32)
    n = a32.size // m32
    r = np.empty(n * out_words, np.uint32)
    rc = lib().orc_gmp_batch(1 if is_add else 0, n, m32, _p(a32), _p(b32), _p(r), out_words, threads)
    if rc != 0:
        raise RuntimeError("GMP (libgmp.so.10) not available")
    return r


def batch_u64(op: str, a: np.ndarray, b: np.ndarray, m: int, threads: int = 1):
    """Multi-threaded restatement (add -> (r, carry); mul -> full product)."""
    a, b = _c(a, np.uint64), _c(b, np.uint64)
    n = a.size // m
    if op == "add":
        r, c = np.empty_like(a), np.empty(n, np.uint8)
        lib().orc_batch_u64(0, n, m, _p(a), _p(b), _p(r), _p(c), threads)
        return r, c
    r = np.empty(n * 2 * m, np.uint64)
    lib().orc_batch_u64(1, n, m, _p(a), _p(b), _p(r), None, threads)
    return r


# --- word formats (GMP mpz_import / mpz_export conventions) ----------------------
#
# A field of `words` words of `size` bytes per instance; `order` 1 = most
# significant word first, -1 = least significant first; `endian` 1 = big-endian
# bytes in a word, -1 or 0 = little-endian (native on every supported host).
# These restate GMP's documented formats; test_oracle.py pins them on GMP itself.

def import_words(src: np.ndarray, n: int, words: int, size: int, order: int, endian: int,
                 limbs: int) -> np.ndarray:
    """Fields of GMP words -> n*limbs u64 limbs (values mod 2^(64*limbs))."""
    b = np.ascontiguousarray(src).view(np.uint8).reshape(n, words, size)
    if order == 1:
        b = b[:, ::-1, :]
    if endian == 1:
        b = b[:, :, ::-1]
    le = np.ascontiguousarray(b).reshape(n, words * size)      # little-endian bytes of each value
    out = np.zeros((n, limbs * 8), np.uint8)
    k = min(limbs * 8, words * size)
    out[:, :k] = le[:, :k]
    return out.view(np.uint64).ravel()


def export_words(src: np.ndarray, n: int, limbs: int, words: int, size: int, order: int, endian: int):
    """n*limbs u64 limbs -> (fields of GMP words as uint8, significant-word counts).
    Values wider than the field keep their low words (the counts say so)."""
    le = np.ascontiguousarray(src, dtype=np.uint64).reshape(n, limbs).view(np.uint8).reshape(n, limbs * 8)
    field = np.zeros((n, words * size), np.uint8)
    k = min(limbs * 8, words * size)
    field[:, :k] = le[:, :k]
    nz = le != 0
    top = np.where(nz.any(axis=1), limbs * 8 - 1 - np.argmax(nz[:, ::-1], axis=1), -1)
    counts = np.where(top >= 0, top // size + 1, 0).astype(np.uint32)
    b = field.reshape(n, words, size)
    if endian == 1:
        b = b[:, :, ::-1]
    if order == 1:
        b = b[:, ::-1, :]
    return np.ascontiguousarray(b).ravel(), counts


def gmp_import(src_field: np.ndarray, words: int, size: int, order: int, endian: int, limbs: int):
    """GMP's mpz_import of one field -> (limbs u64, significant limbs)."""
    f = np.ascontiguousarray(src_field, dtype=np.uint8)
    out = np.zeros(limbs, np.uint64)
    cnt = lib().orc_gmp_import(_p(f), words, order, size, endian, _p(out), limbs)
    if cnt < 0:
        raise RuntimeError("GMP (libgmp.so.10) not available")
    return out, cnt


def gmp_export(x: np.ndarray, words: int, size: int, order: int, endian: int):
    """GMP's mpz_export of one value into a field of `words` words -> (field, count)."""
    x = np.ascontiguousarray(x, dtype=np.uint64)
    field = np.zeros(words * size, np.uint8)
    cnt = lib().orc_gmp_export(_p(x), x.size, order, size, endian, _p(field), words)
    if cnt < 0:
        raise RuntimeError("GMP (libgmp.so.10) not available")
    return field, cnt


# --- pure-Python int cross-oracles (small cases) --------------------------------

def to_ints(x: np.ndarray, m: int) -> list[int]:
    """Instances of a flat little-endian limb array as Python ints."""
    bits = x.dtype.itemsize * 8
    rows = np.ascontiguousarray(x).reshape(-1, m)
    out = []
    for row in rows:
        v = 0
        for limb in reversed(row.tolist()):
            v = (v << bits) | int(limb)
        out.append(v)
    return out


def from_ints(vals: list[int], m: int, dtype=np.uint64) -> np.ndarray:
    bits = np.dtype(dtype).itemsize * 8
    mask = (1 << bits) - 1
    out = np.empty(len(vals) * m, dtype)
    for i, v in enumerate(vals):
        for k in range(m):
            out[i * m + k] = (v >> (bits * k)) & mask
    return out


def py_add(a, b, m):
    bits = a.dtype.itemsize * 8 * m
    xs, ys = to_ints(a, m), to_ints(b, m)
    s = [x + y for x, y in zip(xs, ys)]
    return from_ints([v & ((1 << bits) - 1) for v in s], m, a.dtype), np.array([v >> bits for v in s], np.uint8)


def py_mul(a, b, m, full=True):
    bits = a.dtype.itemsize * 8 * m
    xs, ys = to_ints(a, m), to_ints(b, m)
    prods = [x * y for x, y in zip(xs, ys)]
    if full:
        return from_ints(prods, 2 * m, a.dtype)
    return from_ints([v & ((1 << bits) - 1) for v in prods], m, a.dtype)
