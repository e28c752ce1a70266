"""The C++ drop-in header: a program calling gpuAdd / gpuMultiply /
gpuMulFFT with the reference's shapes compiles against the library and its
results match the oracle."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import PKG, ROOT

pytestmark = pytest.mark.gpu


def read_arrays(path, dtypes):
    out = []
    with open(path, "rb") as f:
        for dt in dtypes:
            n = int(np.frombuffer(f.read(8), np.uint64)[0])
            out.append(np.frombuffer(f.read(n), dt).copy())
    return out


def test_reference_shaped_cpp_callers(lib, tmp_path):
    exe = tmp_path / "compat_main"
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp",
           "compat_main.cpp"), "-o", str(exe), "-L", PKG, "-lmidint_gb300", f"-Wl,-rpath,{PKG}"]
    subprocess.run(cmd, check=True)
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(out)], check=True)
    u64, u32, u16 = np.uint64, np.uint32, np.uint16
    (a, b, r, a2, b2, r2, a3, b3, r3, a4, b4, r4) = read_arrays(out, [u64] * 3 + [u32] * 3 + [u64] * 3 +
                                                               [u16, u16, u32])
    assert np.array_equal(r, O.add(a, b, 64, with_carry=False))
    assert not r[:64].any()                                   # all-ones + 1 wrapped to zero
    assert np.array_equal(r2, O.add(a2, b2, 129, with_carry=False))
    assert np.array_equal(r3, O.mul(a3, b3, 128, full=False))
    n, M = 37, 512
    want = O.mul(a4.view(u32), b4.view(u32), M // 2, full=False)  # low M digits = low M/2 words
    assert np.array_equal(r4.view(u16)[: n * M].view(u32), want)
