"""The C ABI surface, checked without a GPU: every function include/midint.h
declares is exported by libmidint_gb300.so and bound by the Python mirror, and
argument errors come back as MI_EINVAL before any device work."""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

import midint


def declared_functions(header: str) -> list[str]:
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mi_[a-z0-9_A-Z]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions("midint.h")
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_mirror_binds_every_declared_symbol(lib):
    assert sorted(midint.SIGNATURES) == declared_functions("midint.h")


def test_status_strings(lib):
    assert lib.mi_status_string(midint.MI_OK) == b"MI_OK"
    assert lib.mi_status_string(midint.MI_EINVAL).startswith(b"MI_EINVAL")
    assert lib.mi_version() >= 100


def test_argument_errors_need_no_device(lib):
    buf = np.zeros(64, np.uint64)
    p = buf.ctypes.data
    # null buffers, zero limbs, oversize limbs: rejected before touching CUDA
    assert lib.mi_add_u64(None, None, p, p, None, 1, 4, None) == midint.MI_EINVAL
    assert b"null" in lib.mi_last_error()
    assert lib.mi_add_u64(None, p, p, p, None, 1, 0, None) == midint.MI_EINVAL
    assert lib.mi_add_u64(None, p, p, p, None, 1, 1 << 20, None) == midint.MI_EINVAL
    assert lib.mi_mul_full_u64(None, p, p, p + 8, 1, 4, None) == midint.MI_EINVAL  # result overlaps
    assert lib.mi_mul_lo_u32(None, p, p, p, 1, 5000, None) == midint.MI_EINVAL
    assert lib.mi_compat_gpuAdd_u64(-1, 4, p, p, p) == midint.MI_EINVAL
    # a partial overlap of result and operand is refused; exact aliasing is allowed
    assert lib.mi_add_u64(None, p, p, p + 8, None, 2, 4, None) == midint.MI_EINVAL
    assert lib.mi_ctx_set_tuning(None, midint.TUNE_ADD_THREAD_BYTES, 0, 16) == midint.MI_EINVAL
    assert lib.mi_ctx_get_tuning(None, midint.TUNE_PLAIN_NTT_MIN, 0, p) == midint.MI_EINVAL


def test_empty_batch_is_a_no_op(lib):
    buf = np.zeros(8, np.uint64)
    p = buf.ctypes.data
    for f in (lib.mi_mul_lo_u64, lib.mi_mul_full_u64):
        assert f(None, p, p, p + 4096, 0, 4, None) == midint.MI_OK


def test_python_mirror_rejects_bad_host_arrays(lib):
    a = np.zeros(10, np.uint32)
    with pytest.raises(midint.MidintError):
        midint.gpuAdd(midint.U64bits, 4, 2, a, a, a)       # wrong dtype
    b = np.zeros(4, np.uint64)
    with pytest.raises(midint.MidintError):
        midint.gpuMultiply(midint.U64bits, 4, 2, b, b, b)  # too short


def test_context_without_device_reports_enodev(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    h = ctypes.c_void_p()
    st = lib.mi_ctx_create(0, ctypes.byref(h))
    assert st == midint.MI_ENODEV and h.value is None


def test_header_constants_match_the_python_mirror():
    """Every enumerator and numeric #define of include/midint.h that midint.py
    mirrors has the same value there (under its own name or without MI_)."""
    text = open(os.path.join(ROOT, "include", "midint.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    consts = {n: int(v) for n, v in re.findall(r"\b(MI_[A-Z0-9_]+)\s*=\s*(\d+)", text)}
    consts.update({n: int(v) for n, v in re.findall(r"#define\s+(MI_[A-Z0-9_]+)\s+(\d+)u?\b", text)})
    assert "MI_TUNE_LO_NTT_MIN" in consts and "MI_OP_MUL" in consts
    checked = 0
    for name, value in consts.items():
        py = [n for n in (name, name[3:]) if hasattr(midint, n)]
        if not py:
            continue  # a limit the mirror leaves to the C side
        assert getattr(midint, py[0]) == value, name
        checked += 1
    assert checked >= 20
    tunes = [n for n in consts if n.startswith("MI_TUNE_")]
    assert all(hasattr(midint, n[3:]) for n in tunes)
