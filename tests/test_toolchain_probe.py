"""What the CUDA 13.0 toolchain accepts for sm_103a tensor-core instructions.

The exact INT8 Toeplitz form of the classical product would need
`tcgen05.mma ... .kind::i8` (8-bit integer operands, 32-bit integer
accumulators in tensor memory).  ptxas refuses that kind for sm_103a ("not
supported on .target 'sm_103a'") while it accepts it for sm_100a, and accepts
the floating-point `kind::f16` for sm_103a.  So on this GPU the only tensor-core
route to the product would be floating-point arithmetic on integer-valued
digits, which the library excludes (every operation here is integer
arithmetic); the classical product stays on the integer multiply-add pipe.
Needs only nvcc (no GPU)."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"

SRC = r"""
#include <cstdint>
__global__ void k(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
               "tcgen05.mma.cta_group::1.kind::KIND [%0], %1, %2, %3, p;\n}\n"
               :: "r"(taddr), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(taddr));
}
"""


def _compile(tmp_path, kind: str, arch: str):
    src = tmp_path / f"probe_{kind}_{arch}.cu"
    src.write_text(SRC.replace("KIND", kind))
    res = subprocess.run([NVCC, "-gencode", f"arch=compute_{arch},code=sm_{arch}", "-c", str(src),
                          "-o", str(tmp_path / f"probe_{kind}_{arch}.o")], capture_output=True, text=True)
    return res.returncode, res.stdout + res.stderr


@pytest.mark.skipif(not os.path.exists(NVCC), reason="nvcc absent")
def test_int8_tensor_mma_is_not_available_on_sm103a(tmp_path):
    rc, log = _compile(tmp_path, "i8", "103a")
    assert rc != 0 and "not supported on .target 'sm_103a'" in log, log
    rc, log = _compile(tmp_path, "i8", "100a")       # the same instruction on sm_100a assembles
    assert rc == 0, log
    rc, log = _compile(tmp_path, "f16", "103a")      # the floating-point kind assembles on sm_103a
    assert rc == 0, log
