"""Autotuner for the library's launch choices.

Measures, on the GPU it runs on, every candidate of the tunable choices through
the context's tuning override (`mi_ctx_set_tuning`) and writes

  csrc/tuning_table.h   the defaults compiled into the library
  tuning.json           the record: device, every candidate's time, the pick

Knobs:
  * addition, per size class c = ceil(log2(u64 limbs)), c = 0..12: operand bytes
    per thread (16, 32 or 64), on batches of about 256 MiB of operands (twice
    the L2) at the class's largest size;
  * plain classical/NTT crossover of mi_mul_u64: both paths timed on square
    products from 64 to 1024 u64 limbs; the crossover is the smallest measured
    size from which the NTT is faster at every larger measured size;
  * the same for the low half (mi_mul_lo_u64), 256 to 2048 limbs;
  * the same for the fused composite (mi_poly_u64: four classical low halves
    against four low halves on transforms), 64 to 2048 limbs;
  * ragged classical/NTT crossovers: the 200000-op mixed ragged workload (40%
    adds, operand bits log-uniform in [256, 65536]) timed end to end for every
    candidate pair of thresholds (the shorter operand from which every
    product uses the NTT, and the one from which products whose NTT runs on
    40-bit digits and three primes do); the fastest pair wins;
  * host-buffer calls: chunk count of the copy/compute pipeline, or zero-copy
    kernels on mapped pinned buffers, timed on the multiplication batch.

Usage:  python midint-arithmetic_gb300/autotune.py [--out-dir DIR] [--apply]
(--apply writes into the package; otherwise into DIR, default the working
directory, for review.)  Needs a CUDA device.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

L2_BYTES = 129 * 1024 * 1024


def _timer(fn, reps: int, warmup: int, stream) -> float:
    """Median over 3 rounds of the mean device time (ms) of `reps` calls."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    rounds = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        rounds.append(e0.elapsed_time(e1) / reps)
    return float(np.median(rounds))


def tune_add(ctx, stream, dev) -> tuple[list[int], dict]:
    import torch

    import midint

    picks, record = [], {}
    for c in range(13):
        limbs = 1 << c
        n = max(1024, (256 << 20) // (3 * 8 * limbs))
        sets = 2
        a = [torch.randint(-2**62, 2**62, (n * limbs,), dtype=torch.int64, device=dev) for _ in range(sets)]
        b = [torch.randint(-2**62, 2**62, (n * limbs,), dtype=torch.int64, device=dev) for _ in range(sets)]
        r = [torch.empty(n * limbs, dtype=torch.int64, device=dev) for _ in range(sets)]
        cr = [torch.empty(n, dtype=torch.uint8, device=dev) for _ in range(sets)]
        times = {}
        for tb in (16, 32, 64):
            ctx.set_tuning(midint.TUNE_ADD_THREAD_BYTES, c, tb)
            it = [0]

            def step():
                i = it[0] % sets
                it[0] += 1
                ctx.add(a[i], b[i], r[i], n, limbs, carry=cr[i], stream=stream.cuda_stream)

            ms = _timer(step, 20, 5, stream)
            times[tb] = {"ms": ms, "GB/s": n * (3 * 8 * limbs + 1) / (ms * 1e-3) / 1e9}
        best = min(times, key=lambda k: times[k]["ms"])
        ctx.set_tuning(midint.TUNE_ADD_THREAD_BYTES, c, best)
        picks.append(best)
        record[f"class_{c}"] = {"u64_limbs": limbs, "instances": n, "candidates": times, "pick": best}
        del a, b, r, cr
        torch.cuda.empty_cache()
    return picks, record


def crossover_pick(sizes: list[int], ntt_faster: dict[int, bool], never: int = 2049) -> int:
    """The smallest measured size from which the NTT is faster at every larger
    measured size, or `never` when it is not faster at the largest."""
    for i, m in enumerate(sizes):
        if all(ntt_faster[x] for x in sizes[i:]):
            return m
    return never


def tune_plain_crossover(ctx, stream, dev) -> tuple[int, dict]:
    import torch

    sizes = [64, 96, 128, 160, 192, 256, 320, 384, 512, 640, 768, 1024]
    record, ntt_faster = {}, {}
    for m in sizes:
        n = max(512, (64 << 20) // (8 * m))
        a = torch.randint(-2**62, 2**62, (n * m,), dtype=torch.int64, device=dev)
        b = torch.randint(-2**62, 2**62, (n * m,), dtype=torch.int64, device=dev)
        r = torch.empty(2 * n * m, dtype=torch.int64, device=dev)
        sp = stream.cuda_stream
        t_cls = _timer(lambda: ctx.mul_full(a, b, r, n, m, stream=sp), 5, 2, stream)
        t_ntt = _timer(lambda: ctx.mul_ntt(a, b, r, n, m, stream=sp), 5, 2, stream)
        record[str(m)] = {"instances": n, "classical_ns_per_product": t_cls * 1e6 / n,
                          "ntt_ns_per_product": t_ntt * 1e6 / n}
        ntt_faster[m] = t_ntt < t_cls
        del a, b, r
        torch.cuda.empty_cache()
    pick = crossover_pick(sizes, ntt_faster)
    return pick, record


def tune_lo_crossover(ctx, stream, dev) -> tuple[int, dict]:
    """Low-half products, classical (the knob at 2049) against the NTT (the
    knob at 1) through mi_mul_lo_u64, from 256 to 2048 u64 limbs, picked as
    for the plain crossover."""
    import torch

    import midint

    sizes = [256, 320, 384, 448, 512, 640, 768, 1024, 1536, 2048]
    record, ntt_faster = {}, {}
    sp = stream.cuda_stream
    for m in sizes:
        n = max(256, (64 << 20) // (8 * m))
        a = torch.randint(-2**62, 2**62, (n * m,), dtype=torch.int64, device=dev)
        b = torch.randint(-2**62, 2**62, (n * m,), dtype=torch.int64, device=dev)
        r = torch.empty(n * m, dtype=torch.int64, device=dev)
        t = {}
        for name, knob in (("classical", 2049), ("ntt", 1)):
            ctx.set_tuning(midint.TUNE_LO_NTT_MIN, 0, knob)
            t[name] = _timer(lambda: ctx.mul_lo(a, b, r, n, m, stream=sp), 5, 2, stream)
        record[str(m)] = {"instances": n, "classical_ns_per_product": t["classical"] * 1e6 / n,
                          "ntt_ns_per_product": t["ntt"] * 1e6 / n}
        ntt_faster[m] = t["ntt"] < t["classical"]
        del a, b, r
        torch.cuda.empty_cache()
    pick = crossover_pick(sizes, ntt_faster)
    ctx.set_tuning(midint.TUNE_LO_NTT_MIN, 0, pick)
    return pick, record


def tune_poly_crossover(ctx, stream, dev) -> tuple[int, dict]:
    """The fused composite ((a^2 + b)(b^2 + b) + ab) mod 2^(64m) through
    mi_poly_u64, classical (the knob at 2049) against the transform form (the
    knob at 1), from 64 to 2048 u64 limbs, picked as for the plain crossover;
    the two forms' results are compared."""
    import torch

    import midint

    sizes = [64, 96, 128, 160, 192, 256, 320, 384, 448, 512, 640, 768, 1024, 1536, 2048]
    record, ntt_faster = {}, {}
    sp = stream.cuda_stream
    for m in sizes:
        n = max(256, (64 << 20) // (8 * m))
        a = torch.randint(-2**62, 2**62, (n * m,), dtype=torch.int64, device=dev)
        b = torch.randint(-2**62, 2**62, (n * m,), dtype=torch.int64, device=dev)
        r = torch.empty(n * m, dtype=torch.int64, device=dev)
        t, outs = {}, {}
        for name, knob in (("classical", 2049), ("ntt", 1)):
            ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, knob)
            t[name] = _timer(lambda: ctx.poly(a, b, r, n, m, stream=sp), 3, 1, stream)
            outs[name] = r.cpu()
        if not torch.equal(outs["classical"], outs["ntt"]):
            raise SystemExit(f"autotune: the two poly forms differ at {m} limbs")
        record[str(m)] = {"instances": n, "classical_ns_per_instance": t["classical"] * 1e6 / n,
                          "ntt_ns_per_instance": t["ntt"] * 1e6 / n}
        ntt_faster[m] = t["ntt"] < t["classical"]
        del a, b, r
        torch.cuda.empty_cache()
    pick = crossover_pick(sizes, ntt_faster)
    ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, pick)
    return pick, record


def tune_ragged_crossover(ctx, stream, dev, n_ops: int) -> tuple[tuple[int, int], dict]:
    import torch

    import midint
    import workloads

    ops, pool, out_limbs = workloads.ragged_ops(n_ops=n_ops, seed=workloads.SEED_BASE + 3)
    d_ops = torch.from_numpy(ops.view(np.uint8).copy()).to(dev)
    d_in = torch.from_numpy(pool.view(np.int64)).to(dev)
    d_out = torch.empty(out_limbs, dtype=torch.int64, device=dev)
    d_c = torch.empty(n_ops, dtype=torch.uint8, device=dev)
    sb = midint.ragged_scratch_bytes(n_ops)
    scr = torch.empty(sb // 4 + 1, dtype=torch.int32, device=dev)
    sp = stream.cuda_stream
    record = {}
    ref = None
    for th in (64, 96, 112, 128, 144, 160, 192, 257):
        for th40 in (32, 48, 64, 80, 96, 112, 128):
            if th40 >= th and th40 != 32:
                continue  # the same as th40 = th
            ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 0, th)
            ctx.set_tuning(midint.TUNE_RAGGED_NTT_MIN, 1, min(th40, th))
            ms = _timer(lambda: ctx.ragged_run(d_ops, n_ops, d_in, d_out, scr, sb, carry=d_c, stream=sp), 5, 2,
                        stream)
            out = d_out.cpu().numpy()
            if ref is None:
                ref = out.copy()
            elif not np.array_equal(out, ref):
                raise SystemExit(f"autotune: ragged results differ at thresholds {th}, {th40}")
            record[f"{th}/{min(th40, th)}"] = {"ms": ms}
    best = min(record, key=lambda k: record[k]["ms"])
    pick = tuple(int(v) for v in best.split("/"))
    del d_ops, d_in, d_out, d_c, scr
    torch.cuda.empty_cache()
    return pick, {"ops": n_ops, "candidates": record}


def tune_host(ctx) -> tuple[list[int], list[int], list[int], dict]:
    """Host-buffer calls on pinned buffers, wall-clock per call, for every chunk
    count and with zero-copy: class 0 on the addition batch (65536 x 64 u64
    limbs, with carries), class 1 on the classical multiplication batch (16384
    x 128 u64 limbs, full products).  Each class takes its fastest chunk count
    and zero-copy where it beats that; mode 1 is timed with every cap on the
    product kernel's resident blocks per SM (0 = none)."""
    import time

    import torch

    import midint

    def pinned(nwords):
        return torch.randint(-2**62, 2**62, (nwords,), dtype=torch.int64).pin_memory()

    nm, mm, na, ma = 16384, 128, 65536, 64
    ha, hb, hr = pinned(nm * mm), pinned(nm * mm), pinned(2 * nm * mm)
    aa, ab, ar = pinned(na * ma), pinned(na * ma), pinned(na * ma)
    ac = torch.empty(na, dtype=torch.uint8).pin_memory()
    calls = {0: lambda: ctx.host_add(aa, ab, ar, ac, na, ma), 1: lambda: ctx.host_mul_full(ha, hb, hr, nm, mm)}

    def wall(fn, reps=20):
        for _ in range(3):
            fn()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return (time.perf_counter() - t0) / reps * 1e3

    record, chunks, zero_copy, zc_blocks = {}, [], [], []
    for cls, name in ((0, "add"), (1, "mul")):
        cands = {}
        grid = ([(0, c, 0) for c in (2, 3, 4, 6, 8, 12, 16)] + [(1, 1, k) for k in (0, 1, 2, 3)]
                + [(2, c, 0) for c in (2, 3, 4, 6, 8, 12)] + [(3, c, 0) for c in (2, 3, 4, 6, 8, 12)])
        for zc, ch, kb in grid:
            ctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, cls, zc)
            ctx.set_tuning(midint.TUNE_HOST_CHUNKS, cls, ch)
            ctx.set_tuning(midint.TUNE_HOST_ZC_BLOCKS, cls, kb)
            cands[f"zero_copy={zc},chunks={ch},zc_blocks={kb}"] = {"zero_copy": zc, "chunks": ch, "zc_blocks": kb,
                                                                  "ms": wall(calls[cls])}
        # the pipeline's chunk count also serves callers whose buffers are
        # not pinned, so it is the best copy pipeline's unless mode 2 or 3
        # (which chunk the same way) wins
        best_copy = min((v for v in cands.values() if v["zero_copy"] == 0), key=lambda v: v["ms"])
        best = min(cands.values(), key=lambda v: v["ms"])
        zc = best["zero_copy"]
        ch = best["chunks"] if zc in (2, 3) else best_copy["chunks"]
        kb = best["zc_blocks"] if zc == 1 else 0
        ctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, cls, zc)
        ctx.set_tuning(midint.TUNE_HOST_CHUNKS, cls, ch)
        ctx.set_tuning(midint.TUNE_HOST_ZC_BLOCKS, cls, kb)
        chunks.append(ch)
        zero_copy.append(zc)
        zc_blocks.append(kb)
        record[name] = {"candidates": cands, "pick": {"chunks": ch, "zero_copy": zc, "zc_blocks": kb}}
    return chunks, zero_copy, zc_blocks, record


HEADER = """// tuning_table.h -- defaults of the tunable launch choices, written by
// midint-arithmetic_gb300/autotune.py from measurements on {device} ({date}; the
// record of the run is midint-arithmetic_gb300/tuning.json).  Hand edits are
// overwritten by the next tuning run.
#pragma once

#include <cstdint>

namespace mi {{
namespace tuned {{

// mi_mul_u64: square products of at least this many u64 limbs use the NTT.
constexpr uint32_t kPlainNttMin = {plain};
// mi_mul_lo_u64: low halves of products of at least this many u64 limbs come
// from the NTT kernel (2049 = never).
constexpr uint32_t kLoNttMin = {lo};
// mi_poly_u64: composites of at least this many u64 limbs run their four
// products on the NTT (2049 = never).
constexpr uint32_t kPolyNttMin = {poly};
// Ragged runs: products whose shorter operand has at least this many u64
// limbs use the NTT kernel (1..257), and so do those from kRaggedNtt40Min
// limbs whose NTT runs on 40-bit digits and three primes.
constexpr uint32_t kRaggedNttMin = {ragged};
constexpr uint32_t kRaggedNtt40Min = {ragged40};
// Batched addition: bytes of each operand a thread owns (16, 32 or 64), by
// size class c = ceil(log2(u64 limbs)), c = 0..12.
constexpr uint8_t kAddThreadBytes[13] = {{{add}}};
// Host-buffer calls, by operation class {{additions, multiplications}}: chunks a
// large batch is cut into for copy/compute overlap, and the zero-copy mode for
// mapped pinned buffers (0 copies, 1 kernels read and write in place, 2 kernels
// read the operands in place and the results are copied out).
constexpr uint32_t kHostChunks[2] = {{{chunks}}};
constexpr uint32_t kHostZeroCopy[2] = {{{zero_copy}}};
// Zero-copy mode 1: resident blocks per SM of the classical product kernel
// (0: as many as fit).
constexpr uint32_t kHostZcBlocks[2] = {{{zc_blocks}}};

}}  // namespace tuned
}}  // namespace mi
"""


def render_header(device: str, date: str, picks: dict) -> str:
    """csrc/tuning_table.h for the given picks."""
    def join(xs):
        return ", ".join(str(x) for x in xs)

    return HEADER.format(device=device, date=date, plain=picks["plain_ntt_min"], lo=picks["lo_ntt_min"],
                         poly=picks["poly_ntt_min"],
                         ragged=picks["ragged_ntt_min"], ragged40=picks["ragged_ntt40_min"],
                         chunks=join(picks["host_chunks"]),
                         zero_copy=join(picks["host_zero_copy"]), zc_blocks=join(picks["host_zc_blocks"]),
                         add=join(picks["add_thread_bytes"]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out-dir", default=".")
    ap.add_argument("--apply", action="store_true", help="write into the package (csrc/, tuning.json)")
    ap.add_argument("--ragged-ops", type=int, default=200000)
    ap.add_argument("--only", default="add,plain,lo,poly,ragged,host",
                    help="knob groups to measure (others keep the table)")
    args = ap.parse_args()

    import torch

    import midint

    dev = torch.device("cuda:0")
    stream = torch.cuda.Stream(dev)
    ctx = midint.Context(0)
    only = set(args.only.split(","))
    # groups not measured keep the committed record
    with open(os.path.join(HERE, "tuning.json")) as f:
        old = json.load(f)
    picks = dict(old["picks"])
    picks.setdefault("host_chunks", [4, 6])
    picks.setdefault("host_zero_copy", [0, 1])
    picks.setdefault("host_zc_blocks", [0, 0])
    picks.setdefault("lo_ntt_min", 2049)
    picks.setdefault("poly_ntt_min", 2049)
    picks.setdefault("ragged_ntt40_min", picks["ragged_ntt_min"])
    record = {k: old.get(k) for k in ("add", "plain_crossover", "lo_crossover", "poly_crossover", "ragged_crossover",
                                      "host")}
    if "add" in only:
        picks["add_thread_bytes"], record["add"] = tune_add(ctx, stream, dev)
    if "plain" in only:
        picks["plain_ntt_min"], record["plain_crossover"] = tune_plain_crossover(ctx, stream, dev)
    if "lo" in only:
        picks["lo_ntt_min"], record["lo_crossover"] = tune_lo_crossover(ctx, stream, dev)
    if "poly" in only:
        picks["poly_ntt_min"], record["poly_crossover"] = tune_poly_crossover(ctx, stream, dev)
    if "ragged" in only:
        (picks["ragged_ntt_min"], picks["ragged_ntt40_min"]), record["ragged_crossover"] = tune_ragged_crossover(
            ctx, stream, dev, args.ragged_ops)
    if "host" in only:
        picks["host_chunks"], picks["host_zero_copy"], picks["host_zc_blocks"], record["host"] = tune_host(ctx)
    ctx.close()
    device = torch.cuda.get_device_name(0)
    date = datetime.date.today().isoformat()
    header = render_header(device, date, picks)
    record = {"device": device, "date": date, "torch": torch.__version__, "measured": sorted(only),
              "picks": picks, **record}
    if args.apply:
        hpath, jpath = os.path.join(HERE, "csrc", "tuning_table.h"), os.path.join(HERE, "tuning.json")
    else:
        os.makedirs(args.out_dir, exist_ok=True)
        hpath, jpath = os.path.join(args.out_dir, "tuning_table.h"), os.path.join(args.out_dir, "tuning.json")
    with open(hpath, "w") as f:
        f.write(header)
    with open(jpath, "w") as f:
        json.dump(record, f, indent=1)
    print(json.dumps(record["picks"]))


if __name__ == "__main__":
    main()
