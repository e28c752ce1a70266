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
    assert table["kRaggedNttMin"] == picks["ragged_ntt_min"]
    assert table["kAddThreadBytes"] == picks["add_thread_bytes"]
    assert table["kHostChunks"] == picks["host_chunks"]
    assert table["kHostZeroCopy"] == picks["host_zero_copy"]
    assert table["kHostZcBlocks"] == picks["host_zc_blocks"]


def test_picks_are_accepted_values():
    picks = json.load(open(os.path.join(PKG, "tuning.json")))["picks"]
    assert 1 <= picks["plain_ntt_min"] <= 2049
    assert 1 <= picks["lo_ntt_min"] <= 2049
    assert 1 <= picks["ragged_ntt_min"] <= 257
    assert len(picks["add_thread_bytes"]) == 13 and set(picks["add_thread_bytes"]) <= {16, 32, 64}
    assert all(1 <= c <= 64 for c in picks["host_chunks"])
    assert all(0 <= z <= 3 for z in picks["host_zero_copy"])
    assert all(0 <= b <= 3 for b in picks["host_zc_blocks"])
