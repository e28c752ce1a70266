"""Shared test setup: import paths, the `gpu` marker, library build, fixtures."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "midint-arithmetic_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for _p in (ORACLE, PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    """The built C-ABI library (compiled on first use if missing)."""
    import __graft_entry__

    if not os.path.exists(os.path.join(PKG, "libmidint_gb300.so")):
        __graft_entry__.build()
    import midint

    return midint.load()


@pytest.fixture(scope="session")
def ctx(lib):
    import midint

    c = midint.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def dev():
    import torch

    return torch.device("cuda:0")


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name))


class Dev:
    """numpy <-> CUDA tensor helpers that keep the limb bits exactly."""

    @staticmethod
    def put(x: np.ndarray, offset_words: int = 0):
        """Copies x to the GPU; with offset_words > 0 the returned pointer is
        offset into a larger allocation (to test unaligned rows)."""
        import torch

        w = x.view(np.uint32) if x.dtype == np.uint64 else x
        buf = torch.zeros(w.size + offset_words + 4, dtype=torch.int32, device="cuda:0")
        buf[offset_words:offset_words + w.size] = torch.from_numpy(w.view(np.int32).copy()).to("cuda:0")
        return buf, buf.data_ptr() + 4 * offset_words

    @staticmethod
    def empty_words(n32: int, offset_words: int = 0):
        import torch

        buf = torch.full((n32 + offset_words + 4,), -1, dtype=torch.int32, device="cuda:0")
        return buf, buf.data_ptr() + 4 * offset_words

    @staticmethod
    def get(buf, n32: int, offset_words: int = 0, dtype=np.uint64) -> np.ndarray:
        w = buf[offset_words:offset_words + n32].cpu().numpy().view(np.uint32)
        return w.view(dtype).copy()


@pytest.fixture
def devmem():
    return Dev
