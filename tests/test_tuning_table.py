"""The compiled tuning table (csrc/tuning_table.h) holds the picks of the
committed tuning record (tuning.json), and every pick is a value the library
accepts for its knob."""
from __future__ import annotations

import json
import os
import re

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "midint-arithmetic_gb300")


def _table() -> dict:
    src = open(os.path.join(PKG, "csrc", "tuning_table.h")).read()
    out = {}
    for name, dim, body in re.findall(r"constexpr\s+\w+\s+(k\w+)(\[\d+\])?\s*=\s*\{?([^;}]*)\}?;", src):
        vals = [int(v) for v in body.replace(" ", "").split(",") if v]
        out[name] = vals if dim else vals[0]
    return out


def test_table_matches_record():
    table = _table()
    picks = json.load(open(os.path.join(PKG, "tuning.json")))["picks"]
    assert table["kPlainNttMin"] == picks["plain_ntt_min"]
    assert table["kLoNttMin"] == picks["lo_ntt_min"]
    assert table["kPolyNttMin"] == picks["poly_ntt_min"]
    assert table["kRaggedNttMin"] == picks["ragged_ntt_min"]
    assert table["kRaggedNtt40Min"] == picks["ragged_ntt40_min"]
    assert table["kAddThreadBytes"] == picks["add_thread_bytes"]
    assert table["kHostChunks"] == picks["host_chunks"]
    assert table["kHostZeroCopy"] == picks["host_zero_copy"]
    assert table["kHostZcBlocks"] == picks["host_zc_blocks"]


def test_picks_are_accepted_values():
    picks = json.load(open(os.path.join(PKG, "tuning.json")))["picks"]
    assert 1 <= picks["plain_ntt_min"] <= 2049
    assert 1 <= picks["lo_ntt_min"] <= 2049
    assert 1 <= picks["poly_ntt_min"] <= 2049
    assert 1 <= picks["ragged_ntt_min"] <= 257
    assert 1 <= picks["ragged_ntt40_min"] <= picks["ragged_ntt_min"]
    assert len(picks["add_thread_bytes"]) == 13 and set(picks["add_thread_bytes"]) <= {16, 32, 64}
    assert all(1 <= c <= 64 for c in picks["host_chunks"])
    assert all(0 <= z <= 3 for z in picks["host_zero_copy"])
    assert all(0 <= b <= 3 for b in picks["host_zc_blocks"])


def test_crossover_pick_rule():
    import sys

    sys.path.insert(0, PKG)
    from autotune import crossover_pick

    sizes = [64, 128, 256, 512]
    assert crossover_pick(sizes, {64: False, 128: False, 256: True, 512: True}) == 256
    # a faster size below a slower one does not count
    assert crossover_pick(sizes, {64: True, 128: False, 256: True, 512: True}) == 256
    assert crossover_pick(sizes, {64: True, 128: True, 256: True, 512: True}) == 64
    assert crossover_pick(sizes, {64: True, 128: True, 256: True, 512: False}) == 2049


def test_recorded_crossovers_follow_the_rule():
    """The committed picks are what the rule gives on the committed timings."""
    import sys

    sys.path.insert(0, PKG)
    from autotune import crossover_pick

    rec = json.load(open(os.path.join(PKG, "tuning.json")))
    for key, pick in (("plain_crossover", "plain_ntt_min"), ("lo_crossover", "lo_ntt_min")):
        sizes = sorted(int(m) for m in rec[key])
        faster = {m: rec[key][str(m)]["ntt_ns_per_product"] < rec[key][str(m)]["classical_ns_per_product"]
                  for m in sizes}
        assert crossover_pick(sizes, faster) == rec["picks"][pick], key
    poly = rec["poly_crossover"]
    sizes = sorted(int(m) for m in poly)
    faster = {m: poly[str(m)]["ntt_ns_per_instance"] < poly[str(m)]["classical_ns_per_instance"] for m in sizes}
    assert crossover_pick(sizes, faster) == rec["picks"]["poly_ntt_min"]


def test_header_is_what_the_tuner_writes():
    """csrc/tuning_table.h is byte for byte the tuner's template filled with
    the committed record (no hand edits)."""
    import sys

    sys.path.insert(0, PKG)
    import autotune

    rec = json.load(open(os.path.join(PKG, "tuning.json")))
    header = autotune.render_header(rec["device"], rec["date"], rec["picks"])
    assert open(os.path.join(PKG, "csrc", "tuning_table.h")).read() == header
