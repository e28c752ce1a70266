"""One launch of each kernel family on the benchmark's shapes, for profilers.

Runs, on cuda:0, each selected operation once (after one untimed warm-up call
when --warmup 1) with seeded inputs already resident on the device:

  add     65536 x 64 u64 limbs, carries        (k_add)
  add6    6a + 10b on the same batch            (k_add, 6a+10b variant)
  mul     16384 x 128 u64 limbs, full products  (k_mul)
  mul_lo  the same batch, low halves            (k_mul_lo)
  poly    the same batch                        (k_poly)
  ntt     1024 x 1024 u64 limbs                 (k_ntt_mul, 64-bit digits on five primes)
  ntt48   1024 x 768 u64 limbs                  (k_ntt_mul, 48-bit digits on four primes, L = 2048)
  ragged  a mixed ragged list (--ragged-ops)    (k_classify, k_scan, k_scatter, k_rg_*)
  wide    16 pairs x 2^21 u64 limbs             (k_add_wide)
  convert the addition batch to big-endian 8-byte words and back (k_export, k_count_words, k_import)
  ragged_bands  the --ragged-ops list cut into its additions and its products
          by shorter-operand band, each band timed alone as its own captured
          ragged run (CUDA events over 10 replays after 3) and printed as JSON
  ntt_sizes  NTT products at 384/400, 768/800 and 1536/1600 limbs (the first of
          each pair takes 48-bit digits on four primes, the second 64-bit
          digits on five, at the same transform length), ns per product with
          CUDA events over 10 launches after 3, printed as JSON
  ntt_batches  NTT products of 1024 u64 limbs in batches of 152..2736
          instances (the persistent grid holds 3 groups per SM), ms per
          launch with CUDA events over 20 launches after 3 on 3 rotating
          operand sets, printed as JSON
  wide_variants  additions of 16 pairs x 2^21 u64 limbs with no all-ones pair,
          every 8th pair all-ones + 1, and every pair all-ones + 1 (the
          carry runs through every tile), each timed with CUDA events over
          10 launches after 3 and printed as JSON with GB/s

Usage: python midint-arithmetic_gb300/profcase.py [--ops add,mul,...] [--warmup 0|1]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ops", default="add,add6,mul,mul_lo,poly,ntt,ragged,wide,convert")
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--ragged-ops", type=int, default=20000)
    args = ap.parse_args()

    import torch

    import midint
    import workloads

    dev = torch.device("cuda:0")
    ctx = midint.Context(0)
    sp = torch.cuda.current_stream().cuda_stream

    def dput(x):
        return torch.from_numpy(x.view(np.int64)).to(dev)

    calls = []
    ops = args.ops.split(",")
    if "add" in ops or "add6" in ops or "convert" in ops:
        a, b = workloads.add_pairs(n=65536, m=64)
        da, db = dput(a), dput(b)
        dr = torch.empty_like(da)
        dc = torch.empty(65536, dtype=torch.uint8, device=dev)
        if "add" in ops:
            calls.append(lambda: ctx.add(da, db, dr, 65536, 64, carry=dc, stream=sp))
        if "add6" in ops:
            calls.append(lambda: ctx.add6(da, db, dr, 65536, 64, stream=sp))
        if "convert" in ops:
            cw = torch.empty(65536, dtype=torch.int32, device=dev)
            calls.append(lambda: ctx.export_words(da, 65536, 64, dr, 64, 8, 1, 1, counts=cw, stream=sp))
            calls.append(lambda: ctx.import_words(dr, 65536, 64, 8, 1, 1, db, 64, stream=sp))
    if any(o in ops for o in ("mul", "mul_lo", "poly")):
        a, b = workloads.mul_pairs(n=16384, m=128)
        ma, mb = dput(a), dput(b)
        mr = torch.empty(2 * a.size, dtype=torch.int64, device=dev)
        if "mul" in ops:
            calls.append(lambda: ctx.mul_full(ma, mb, mr, 16384, 128, stream=sp))
        if "mul_lo" in ops:
            calls.append(lambda: ctx.mul_lo(ma, mb, mr, 16384, 128, stream=sp))
        if "poly" in ops:
            calls.append(lambda: ctx.poly(ma, mb, mr, 16384, 128, stream=sp))
    if "ntt" in ops:
        a, b = workloads.ntt_pairs(n=1024, m=1024)
        na, nb = dput(a), dput(b)
        nr = torch.empty(2 * a.size, dtype=torch.int64, device=dev)
        calls.append(lambda: ctx.mul_ntt(na, nb, nr, 1024, 1024, stream=sp))
    if "ntt48" in ops:
        a4, b4 = workloads.ntt_pairs(n=1024, m=768)
        qa, qb = dput(a4), dput(b4)
        qr = torch.empty(2 * a4.size, dtype=torch.int64, device=dev)
        calls.append(lambda: ctx.mul_ntt(qa, qb, qr, 1024, 768, stream=sp))
    if "wide" in ops:
        wa, wb = workloads.add_pairs(n=16, m=1 << 21, worst_every=8)
        xa, xb = dput(wa), dput(wb)
        xr = torch.empty_like(xa)
        xc = torch.empty(16, dtype=torch.uint8, device=dev)
        calls.append(lambda: ctx.add(xa, xb, xr, 16, 1 << 21, carry=xc, stream=sp))
    if "ragged" in ops:
        rops, pool, out_limbs = workloads.ragged_ops(n_ops=args.ragged_ops)
        d_ops = torch.from_numpy(rops.view(np.uint8).copy()).to(dev)
        d_in = dput(pool)
        d_out = torch.empty(out_limbs, dtype=torch.int64, device=dev)
        d_c = torch.empty(rops.size, dtype=torch.uint8, device=dev)
        sb = midint.ragged_scratch_bytes(rops.size)
        scr = torch.empty(sb // 4 + 1, dtype=torch.int32, device=dev)
        calls.append(lambda: ctx.ragged_run(d_ops, rops.size, d_in, d_out, scr, sb, carry=d_c, stream=sp))
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        for c in calls:
            c()
    torch.cuda.synchronize()
    for c in calls:
        c()
    torch.cuda.synchronize()
    if "ragged_bands" in ops:
        print(json.dumps(ragged_bands(ctx, dev, sp, args.ragged_ops), indent=1))
    if "wide_variants" in ops:
        print(json.dumps(wide_variants(ctx, dev, sp), indent=1))
    if "ntt_sizes" in ops:
        print(json.dumps(ntt_sizes(ctx, dev, sp), indent=1))
    if "ntt_batches" in ops:
        print(json.dumps(ntt_batches(ctx, dev, sp), indent=1))
    ctx.close()
    print("profcase: ran", ",".join(ops))


def ntt_sizes(ctx, dev, sp) -> dict:
    """ns per NTT product at sizes either side of the 48-bit digit limit."""
    import torch

    import workloads

    res = {}
    for m in (384, 400, 768, 800, 1536, 1600):
        n = 2048 * 1024 // m  # about 2^21 limbs per operand array
        a, b = workloads.ntt_pairs(n=n, m=m)
        da = torch.from_numpy(a.view(np.int64)).to(dev)
        db = torch.from_numpy(b.view(np.int64)).to(dev)
        dr = torch.empty(2 * a.size, dtype=torch.int64, device=dev)
        for _ in range(3):
            ctx.mul_ntt(da, db, dr, n, m, stream=sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            ctx.mul_ntt(da, db, dr, n, m, stream=sp)
        e1.record()
        e1.synchronize()
        res[str(m)] = {"instances": n, "ns_per_product": e0.elapsed_time(e1) / 10 * 1e6 / n}
        del da, db, dr
        torch.cuda.empty_cache()
    return res


def _event_ms(fn, warmup: int, reps: int) -> float:
    """Mean ms per call of fn(i) with CUDA events on the current stream (the
    stream `sp` of the callers)."""
    import torch

    for i in range(warmup):
        fn(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(reps):
        fn(i)
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def ntt_batches(ctx, dev, sp) -> dict:
    import torch

    import workloads

    m, sets = 1024, 3
    a, b = workloads.ntt_pairs(n=2736, m=m)
    da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(sets)]
    db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(sets)]
    dr = [torch.empty(2 * a.size, dtype=torch.int64, device=dev) for _ in range(sets)]
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    out = {}
    for n in (152, 304, 456, 608, 760, 912, 1024, 1368, 1824, 2736):
        ms = _event_ms(lambda i: ctx.mul_ntt(da[i % sets], db[i % sets], dr[i % sets], n, m, stream=sp), 3, 20)
        out[str(n)] = {"ms": ms, "us_per_instance_per_sm": ms * 1e3 * sms / n}
    return out


def wide_variants(ctx, dev, sp) -> dict:
    """16 x 2^21-limb additions with 0, 1/8 and all pairs carrying through."""
    import torch

    import workloads

    n, m = 16, 1 << 21
    res = {}
    for name, worst in (("uniform", 0), ("every 8th all-ones", 8), ("all all-ones", 1)):
        a, b = workloads.add_pairs(n=n, m=m, worst_every=worst)
        da = torch.from_numpy(a.view(np.int64)).to(dev)
        db = torch.from_numpy(b.view(np.int64)).to(dev)
        dr = torch.empty_like(da)
        dc = torch.empty(n, dtype=torch.uint8, device=dev)
        for _ in range(3):
            ctx.add(da, db, dr, n, m, carry=dc, stream=sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            ctx.add(da, db, dr, n, m, carry=dc, stream=sp)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / 10
        res[name] = {"ms": ms, "GB/s": (3 * n * m * 8 + n) / ms / 1e6}
        del da, db, dr
        torch.cuda.empty_cache()
    res["device_status"] = ctx.device_status()
    return res


# (name, kind, lowest shorter-operand limbs, highest) of each band
BANDS = (("adds", 0, 1, 1024), ("mul 1..8", 1, 1, 8), ("mul 9..16", 1, 9, 16), ("mul 17..32", 1, 17, 32),
         ("mul 33..64", 1, 33, 64), ("mul 65..127", 1, 65, 127), ("mul >=128", 1, 128, 1024))


def ragged_bands(ctx, dev, sp, n_ops: int) -> dict:
    """Each band of the ragged list run alone: ops, ms per run and the
    32x32-bit partial products of the classical product per second."""
    import torch

    import midint
    import workloads

    rops, _, _ = workloads.ragged_ops(n_ops=n_ops)
    kind, la, lb = rops["kind"], rops["la"], rops["lb"]
    short = np.minimum(la, lb)
    res = {}
    for name, k, lo, hi in (("all", -1, 1, 1024),) + BANDS:
        sel = (short >= lo) & (short <= hi) & ((kind == k) if k >= 0 else True)
        o, pool, out_limbs = workloads.pack_ops(kind[sel].astype(np.uint32), la[sel].astype(np.uint32),
                                                lb[sel].astype(np.uint32), workloads.SEED_BASE + 5)
        d_ops = torch.from_numpy(o.view(np.uint8).copy()).to(dev)
        d_in = torch.from_numpy(pool.view(np.int64)).to(dev)
        d_out = torch.empty(out_limbs, dtype=torch.int64, device=dev)
        d_c = torch.empty(o.size, dtype=torch.uint8, device=dev)
        sb = midint.ragged_scratch_bytes(o.size)
        scr = torch.empty(sb // 4 + 1, dtype=torch.int32, device=dev)
        g = ctx.ragged_graph(d_ops, o.size, d_in, d_out, scr, sb, carry=d_c)
        for _ in range(3):
            g.launch(sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            g.launch(sp)
        e1.record()
        e1.synchronize()
        g.close()
        ms = e0.elapsed_time(e1) / 10
        pp = int((4 * la[sel].astype(np.int64) * lb[sel].astype(np.int64) * (kind[sel] == 1)).sum())
        res[name] = {"ops": int(sel.sum()), "ms": ms, "G_pp_per_s": pp / ms / 1e6}
    return res


if __name__ == "__main__":
    main()
