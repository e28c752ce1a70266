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


def test_instance_ranges_are_slices_of_one_batch():
    import workloads

    a0, b0 = workloads.mul_pairs(n=8, m=3)
    a1, b1 = workloads.mul_pairs(n=3, m=3, first=5)
    assert (a1 == a0[15:24]).all() and (b1 == b0[15:24]).all()
    x0, y0 = workloads.add_pairs(n=24, m=2)
    x1, y1 = workloads.add_pairs(n=10, m=2, first=13)         # worst-case rows stay at global index % 8 == 0
    assert (x1 == x0[26:46]).all() and (y1 == y0[26:46]).all()
    n0, _ = workloads.ntt_pairs(n=40, m=2)
    n1, _ = workloads.ntt_pairs(n=20, m=2, first=17)
    assert (n1 == n0[34:74]).all()


def test_targets_object_is_compact_and_complete():
    out = {"roofline": {"frac": 0.7462053}, "ms_per_step": 0.147008,
           "e2e": {"frac_link": 0.61234, "link_gbs": 311.23}}
    extra = {"add_4096bit": {"roofline": {"frac": 0.9231}, "ms_per_launch": 0.0161234},
             "ntt_mul_65536bit": {"roofline": {"frac": 0.731}, "ms_per_launch": 0.0989},
             "ragged_200k": {"ragged_vs_plain": 2.5234, "ragged_ms": 1.7171, "results_identical": True},
             "serving": {"fixed_load": {"offered_req/s": 4000.0,
                                        "batched": {"p50_ms": 0.2612, "p99_ms": 0.5512},
                                        "per_request": {"p50_ms": 0.9, "p99_ms": 3.1}}}}
    t = bench.targets(out, extra)
    assert t["add_4096bit"]["frac_hbm"] == 0.9231 and t["add_4096bit"]["target"] == 0.80
    assert t["ragged"]["vs_plain"] == 2.523 and t["ragged"]["results_identical"] is True
    assert t["serving"]["batched_p50_p99_ms"] == [0.261, 0.551]
    assert t["ntt_mul_65536bit"]["frac"] == 0.731 and t["mul_8192bit"]["frac"] == 0.7462
    import json
    assert len(json.dumps(t)) < 700                          # fits the end of a kept output tail
