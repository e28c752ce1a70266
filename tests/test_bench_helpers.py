"""bench.py's pure helpers, on CPU: whole-job rates and the HBM position of
the headline kernel."""
from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_job_rate_counts_every_rank():
    assert bench.job_rate(1, 16384, 0.5) == 16384 / 0.5e-3
    assert bench.job_rate(4, 16384, 0.5) == 4 * 16384 / 0.5e-3


def test_hbm_position():
    pos = bench.hbm_position(4 * (16 << 20), 0.1464, 6767.7)
    assert pos["unit"] == "GB/s" and pos["bytes_per_launch"] == 64 << 20
    assert abs(pos["achieved"] - (64 << 20) / 0.1464e-3 / 1e9) < 1e-9
    assert 0.06 < pos["frac"] < 0.08  # the product kernel moves 64 MiB in 0.15 ms: far from HBM-bound
    assert bench.hbm_position(1 << 20, 1.0, None)["frac"] is None
