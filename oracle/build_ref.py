"""Compiles the reference's own CPU path into oracle/_ref/libref.so.

Recipe: g++ on oracle/ref/ref_driver.cpp, which includes the reference's
cuda/helper.h from the reference tree in place (never copied), against the
GMP declaration shim oracle/ref/gmp.h and the installed libgmp.so.10; helper.h
also names cudaGetErrorString, so libcudart is linked.  Outputs go only to
oracle/_ref/.  Needs the reference tree: its cuda/ directory is
$MIDINT_REFERENCE_CUDA when that is set, else the reference checkout this
recipe was written against; returns None when neither exists (the GPU
machines have no copy of it and use the restatement in orc.c instead).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_CUDA = os.environ.get("MIDINT_REFERENCE_CUDA", "/root/reference/cuda")
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "libref.so")
CUDA = "/usr/local/cuda"


def build(force: bool = False) -> str | None:
    if not os.path.exists(os.path.join(REF_CUDA, "helper.h")):
        return None
    src = os.path.join(HERE, "ref", "ref_driver.cpp")
    deps = [src, os.path.join(HERE, "ref", "gmp.h"), os.path.join(REF_CUDA, "helper.h")]
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-w",
           "-I", os.path.join(HERE, "ref"), "-I", REF_CUDA, "-I", os.path.join(CUDA, "include"),
           src, "-o", OUT, "-l:libgmp.so.10", "-L", os.path.join(CUDA, "lib64"), "-lcudart"]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
