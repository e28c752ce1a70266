"""Benchmark of the GB300 batched big-integer library (one JSON line on rank 0).

Headline workload: plain classical multiplication, 16384 pairs of 8192-bit
integers (128 u64 limbs) -> 16384-bit full products, uniform seeded limbs.
A step is one batched multiplication over the whole batch.

  value : products/s with operands resident in HBM; K launches on rotating
          operand sets whose total (4 x 64 MiB) exceeds the 129 MB L2, timed
          with CUDA events on the launching stream.
  e2e   : the same metric through the C ABI's host-buffer call
          (mi_host_mul_full_u64) from pinned host memory to pinned host
          memory, every byte crossing the host link inside the timed region
          (the tuned path: zero-copy kernels for multiplications; the copy
          pipeline's time is reported beside it).
  roofline: the multiplication kernel against the integer-multiply ceiling
          measured in-process (mi_calib_mul32_peak), in 32x32-bit partial
          products/s; 65536 partial products per instance.
  workloads: the other benchmark rows measured in the same run (addition GB/s
          and %HBM against MEASURED_PEAKS.json, the u32-limb variant).
  cpu_baseline: the oracle's port of the reference CPU path (GMP mpz_mul via
          gmpAddMulOnce, all host cores) on a bounded sample.

`--impl reference` times the reference's CPU implementation of the path (the
oracle's port of gmpAddMulOnce over GMP; the reference's own build cannot run
on an Arm GPU host) on the same workload with all host threads.

Multi-GPU (N>1): one rank per GPU under torchrun (`--gpus N` without a
launcher re-executes itself under torch.distributed.run).  Every rank
multiplies its own contiguous range of the job's instances (instances are
independent, no collective on the data path); the ragged list of the whole
job is split across ranks by estimated work; max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "midint-arithmetic_gb300"))

import numpy as np  # noqa: E402

METRIC = "add GB/s (%HBM); mul products/s by size, ragged-batched vs plain; p50/p99 ms"
N_MUL, M_MUL = 16384, 128
N_ADD, M_ADD = 65536, 64
L2_BYTES = 129 * 1024 * 1024
CHECK_N = 256  # instances of the timed batch cross-checked against the CPU baseline
SERVE_FIXED_RATE = 4000.0  # requests/s: the serving row's fixed offered load


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-extra", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--cpu-seconds", type=float, default=6.0, help="CPU-baseline sample budget")
    ap.add_argument("--ragged-ops", type=int, default=200000, help="ops in the ragged batch")
    ap.add_argument("--case", default=None,
                    help="profiling cases instead of the bench (comma list; see run_case): one launch of each "
                         "named kernel family, or a timing scan")
    ap.add_argument("--case-warmup", type=int, default=1, help="untimed calls before a case's launches")
    ap.add_argument("--case-ragged-ops", type=int, default=20000, help="ops in the ragged case's list")
    ap.add_argument("--sections", default="add,ntt,ragged,serving,u32,fused,wide",
                    help="secondary workloads to run (comma list of add, ntt, ragged, serving, u32, fused, wide; "
                         "sweep, the reference driver's size sweep, runs only when named)")
    return ap.parse_args()


# --- distributed plumbing ------------------------------------------------------

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_dist(world, local):
    import torch

    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local)
        dist.init_process_group(backend="nccl")
    else:
        torch.cuda.set_device(0)


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    """The largest x over all ranks (a step time: the job ends with its slowest rank)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seed(base: int, rank: int) -> int:
    """Seed of a rank's own batch: ranks process disjoint instances (weak scaling)."""
    return base + 1000 * rank


def instance_range(n_per_rank: int, rank: int) -> tuple[int, int]:
    """The instances [lo, hi) of the whole job's batch that a rank processes:
    contiguous ranges of equal size (instances are independent, so the batch
    shards without any exchange)."""
    return rank * n_per_rank, (rank + 1) * n_per_rank


def launch_command(args_argv: list[str], gpus: int, port: int) -> list[str]:
    """The torchrun command that runs this bench with one rank per GPU of one
    node; the ranks read RANK / LOCAL_RANK / WORLD_SIZE from the environment."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
            "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__), *args_argv]


def check_world(gpus: int, world: int) -> str | None:
    """'launch' when --gpus asks for more ranks than the environment has and
    no launcher started this process; an error message when a launcher
    started a different number of ranks; None when they agree."""
    if gpus == world:
        return None
    if world == 1 and "WORLD_SIZE" not in os.environ:
        return "launch"
    return f"--gpus {gpus} but the launcher started {world} ranks"


def ragged_work_estimate(kind: np.ndarray, la: np.ndarray, lb: np.ndarray) -> np.ndarray:
    """Estimated device seconds of each ragged op, for splitting a list across
    ranks: additions move 3 x 8 bytes per limb at about 6.5 TB/s; products
    cost the cheaper of the classical form (4 la lb partial products at about
    7e12/s) and an NTT of the next power of two of la + lb u64 digits (about
    97 ns per 2048-point product, scaled by L log L)."""
    la = la.astype(np.float64)
    lb = lb.astype(np.float64)
    add = 24.0 * np.maximum(la, lb) / 6.5e12
    L = np.maximum(256.0, 2.0 ** np.ceil(np.log2(la + lb)))
    ntt = 97e-9 * (L / 2048.0) * (np.log2(L) / 11.0)
    mul = np.minimum(4.0 * la * lb / 7e12, ntt)
    return np.where(kind == 0, add, mul)


def shard_ragged(work: np.ndarray, world: int) -> list[np.ndarray]:
    """Splits a ragged list across ranks by estimated work: ops in descending
    cost are dealt to ranks in snake order (0..w-1, w-1..0, ...), so every
    rank gets about the same total; each rank's indices come back in list
    order.  Every op lands on exactly one rank."""
    order = np.argsort(-work, kind="stable")
    pos = np.arange(order.size) % (2 * world)
    owner = np.where(pos < world, pos, 2 * world - 1 - pos)
    return [np.sort(order[owner == r]) for r in range(world)]


def job_rate(world: int, units_per_rank: int, max_ms: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank / (max_ms * 1e-3)


def hbm_position(bytes_per_launch: int, ms: float, peak_gbs) -> dict:
    """Where a launch that moves `bytes_per_launch` in `ms` sits against the
    measured HBM bandwidth (for kernels bound elsewhere: shows the distance)."""
    gbs = bytes_per_launch / (ms * 1e-3) / 1e9
    return {"achieved": gbs, "peak": peak_gbs, "unit": "GB/s", "bytes_per_launch": bytes_per_launch,
            "frac": (gbs / peak_gbs) if peak_gbs else None}


# --- clocks ----------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi sampling (200 ms) of SM clocks and throttle reasons."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[3:7]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


# --- CPU baseline (oracle port of the reference CPU path) -------------------------

def cpu_baseline(a: np.ndarray, b: np.ndarray, m: int, budget_s: float, op: str = "mul",
                 check: np.ndarray | None = None) -> dict:
    """GMP via the oracle's port of gmpAddMulOnce on all host cores, repeated
    over growing prefixes of the batch until about budget_s of wall time.
    With `check` (the GPU's products of the first instances) the first CPU
    pass is also compared with it, limb for limb."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    threads = os.cpu_count() or 1
    n = a.size // m
    a32, b32 = a.view(np.uint32), b.view(np.uint32)
    m32 = 2 * m
    out_words = m32 if op == "add" else 2 * m32
    if oracle.gmp_available():
        kind_note = "GMP mpz_%s through the oracle's port of gmpAddMulOnce (cuda/helper.h:146-170)" % op
        run = lambda k: oracle.gmp_batch(op == "add", a32[: k * m32], b32[: k * m32], m32, out_words, threads)
    else:
        kind_note = "oracle C restatement (GMP absent on this host)"
        run = lambda k: oracle.batch_u64(op, a[: k * m], b[: k * m], m, threads)
    k = min(n, CHECK_N)
    done, elapsed = 0, 0.0
    matches = None
    while elapsed < budget_s:
        t0 = time.perf_counter()
        res = run(k)
        dt = time.perf_counter() - t0
        if check is not None and matches is None:
            cpu = np.asarray(res[0] if isinstance(res, tuple) else res).view(np.uint64)[: check.size]
            matches = bool(np.array_equal(cpu, check))
        done += k
        elapsed += dt
        if dt < budget_s / 8 and k < n:
            k = min(n, k * 2)
    out = {"value": done / elapsed, "cores": threads, "kind": "port",
            "sample": f"{done} instances of the workload (prefixes of the batch, repeated), {elapsed:.1f} s; "
                      + kind_note}
    if check is not None:
        out["matches_gpu_first_instances"] = matches
    return out


# --- GPU measurement helpers -------------------------------------------------------

def time_device(fn, sets: int, steps: int, warmup: int, stream) -> float:
    """Average ms per step: warm-up, then `steps` calls on rotating sets,
    bracketed by synchronize + events on the launching stream."""
    import torch

    for i in range(warmup):
        fn(i % sets)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        fn(i % sets)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def measured_peaks() -> dict:
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def link_rates(dev, in_bufs: list[int], out_bufs: list[int], reps: int = 10) -> dict:
    """Host-link rates with pinned host memory: one cudaMemcpyAsync per
    buffer (the sizes of the e2e step's own operand and result buffers),
    host->device alone, device->host alone, and both directions at once on
    two streams.  GB/s of bytes moved, best of `reps`, CUDA events."""
    import torch

    h_in = [torch.empty(n, dtype=torch.uint8).pin_memory() for n in in_bufs]
    d_in = [torch.empty(n, dtype=torch.uint8, device=dev) for n in in_bufs]
    h_out = [torch.empty(n, dtype=torch.uint8).pin_memory() for n in out_bufs]
    d_out = [torch.empty(n, dtype=torch.uint8, device=dev) for n in out_bufs]
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(h2d: bool, d2h: bool) -> float:
        best = float("inf")
        for _ in range(reps + 2):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s1)
            s2.wait_event(e0)
            if h2d:
                with torch.cuda.stream(s1):
                    for d, h in zip(d_in, h_in):
                        d.copy_(h, non_blocking=True)
            if d2h:
                with torch.cuda.stream(s2):
                    for h, d in zip(h_out, d_out):
                        h.copy_(d, non_blocking=True)
            s1.wait_stream(s2)
            e1.record(s1)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    bi, bo = sum(in_bufs), sum(out_bufs)
    t_in, t_out, t_both = timed(True, False), timed(False, True), timed(True, True)
    out = {"h2d_gbs": bi / (t_in * 1e-3) / 1e9, "d2h_gbs": bo / (t_out * 1e-3) / 1e9,
           "both_gbs": (bi + bo) / (t_both * 1e-3) / 1e9, "both_ms": t_both,
           "how": f"pinned cudaMemcpyAsync, one per buffer ({len(in_bufs)} x {in_bufs[0] >> 20} MiB in, "
                  f"{len(out_bufs)} x {out_bufs[0] >> 20} MiB out), best of {reps}, CUDA events"}
    # the same link streamed by the SMs over mapped pinned memory, as the
    # zero-copy calls use it (mi_calib_host_link): reads, writes, and a copy
    # of half the bytes each way; the faster of the two both-ways rates is the
    # end-to-end denominator
    try:
        import midint

        nb = bi + bo
        src = torch.empty(nb, dtype=torch.uint8).pin_memory()
        dst = torch.empty(nb, dtype=torch.uint8).pin_memory()
        r, w, both = midint.calib_host_link(src, dst, nb)
        out.update({"sm_read_gbs": r, "sm_write_gbs": w, "sm_both_gbs": both,
                    "sm_how": f"SM loads/stores over {nb >> 20} MiB of mapped pinned memory (both ways: "
                              f"{nb >> 21} MiB each), best of 5, CUDA events"})
    except Exception as e:  # noqa: BLE001 -- the calibration is optional, the copy-engine rates stand
        out["sm_error"] = str(e)
    out["best_both_gbs"] = max(out["both_gbs"], out.get("sm_both_gbs", 0.0))
    return out


def run_ours(args):
    import torch

    import midint
    import workloads

    world, rank, local = dist_env()
    init_dist(world, local)
    dev = torch.device("cuda", torch.cuda.current_device())
    ctx = midint.Context(torch.cuda.current_device())
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    # --- headline: classical multiplication, device-resident operands ---------
    a, b = workloads.mul_pairs(n=N_MUL, m=M_MUL, first=instance_range(N_MUL, rank)[0])
    in_bytes = a.nbytes
    set_bytes = 2 * in_bytes + 2 * in_bytes
    sets = max(2, -(-4 * L2_BYTES // set_bytes))
    with torch.cuda.stream(stream):
        da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(sets)]
        db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(sets)]
        dr = [torch.empty(2 * a.size, dtype=torch.int64, device=dev) for _ in range(sets)]
    torch.cuda.synchronize()

    def mul_step(i):
        ctx.mul_full(da[i], db[i], dr[i], N_MUL, M_MUL, stream=sp)

    # results of the first instances, checked later in the CPU-baseline leg
    mul_step(0)
    torch.cuda.synchronize()
    got = dr[0][: CHECK_N * 2 * M_MUL].cpu().numpy().view(np.uint64).copy()

    peak_prod = midint.calib_mul32_peak()
    clocks = ClockSampler(local)
    barrier(world)
    clocks.start()
    time.sleep(0.3)
    ms = time_device(mul_step, sets, args.steps, args.warmup, stream)
    clk = clocks.stop()
    ms = max_over_ranks(world, ms)
    products_s = job_rate(world, N_MUL, ms)
    prods32_per_inst = (2 * M_MUL) ** 2
    achieved_prod = N_MUL * prods32_per_inst / (ms * 1e-3)

    # --- e2e through the host-buffer C-ABI call, pinned host memory ------------
    ha = torch.from_numpy(a.view(np.int64)).pin_memory()
    hb = torch.from_numpy(b.view(np.int64)).pin_memory()
    hr = torch.empty(2 * a.size, dtype=torch.int64).pin_memory()
    han, hbn, hrn = ha.numpy(), hb.numpy(), hr.numpy()
    for _ in range(2):
        ctx.host_mul_full(han, hbn, hrn, N_MUL, M_MUL)
    barrier(world)
    e2e_steps = max(3, min(args.steps, 20))

    def host_steps() -> float:
        hrn[:] = 0
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ctx.host_mul_full(han, hbn, hrn, N_MUL, M_MUL)
        dt = (time.perf_counter() - t0) / e2e_steps
        if not np.array_equal(hrn.view(np.uint64)[: CHECK_N * 2 * M_MUL], got):
            raise SystemExit("bench: e2e product differs from the device-resident one")
        return dt

    zero_copy = ctx.get_tuning(midint.TUNE_HOST_ZERO_COPY, 1)
    e2e_s = max_over_ranks(world, host_steps())
    # the copy pipeline alone, for reference (the tuned default is above)
    ctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 1, 0)
    copy_s = max_over_ranks(world, host_steps())
    ctx.set_tuning(midint.TUNE_HOST_ZERO_COPY, 1, zero_copy)
    path = {0: "mi_host_mul_full_u64 on pinned host buffers; chunked copy-in / compute / copy-out pipeline",
            1: "mi_host_mul_full_u64 on pinned host buffers; the kernel reads the operands and writes the products "
               "in place over the host link (zero-copy, the tuned choice for multiplications)",
            2: "mi_host_mul_full_u64 on pinned host buffers; the kernels read the operands in place over the host "
               "link while the products of earlier chunks are copied out (the tuned choice for multiplications)"
            }[zero_copy]
    # the link's own rate on the step's buffers: the floor of an end-to-end step
    link = link_rates(dev, [in_bytes, in_bytes], [2 * in_bytes])
    e2e = {"value": world * N_MUL / e2e_s, "unit": "products/s", "h2d_bytes_per_step": 2 * in_bytes,
           "d2h_bytes_per_step": 2 * in_bytes, "ms_per_step": e2e_s * 1e3, "path": path,
           "copy_pipeline_ms_per_step": copy_s * 1e3,
           # bytes across the link per step over the step time, against both directions busy at once
           "link_gbs": link["best_both_gbs"], "frac_link": (4 * in_bytes) / e2e_s / 1e9 / link["best_both_gbs"],
           "link": link}
    del da, db, dr
    torch.cuda.empty_cache()

    extra = {}
    if not args.no_extra:
        extra = secondary_workloads(args, ctx, dev, stream, world, rank)

    out = {
        "metric": METRIC,
        "value": products_s,
        "unit": "products/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 limbs (32x32->64-bit integer multiply-add with carry), exact",
        "data": "synthetic: seeded splitmix64 limbs (uniform)",
        "config": {"workload": "plain classical multiplication, 16384 pairs x 8192-bit (128 u64 limbs) -> "
                               "16384-bit full product", "instances_per_gpu": N_MUL, "limbs_u64": M_MUL,
                   "parallelism": f"replicas x{world} (independent instances)",
                   "l2": f"inputs rotate over {sets} operand sets of {set_bytes >> 20} MiB (> 4x L2)"},
        "roofline": {"bound": "int-mul", "achieved": achieved_prod / 1e9, "peak": peak_prod / 1e9,
                     "unit": "G 32x32-bit partial products/s", "frac": achieved_prod / peak_prod,
                     # dram__bytes_read.sum + dram__bytes_write.sum of one k_mul<32> launch (ncu, cold, single
                     # launch): the 32 MiB of operands read once, the product still in L2 at kernel end
                     "traffic": 33.62e6 + 0.23e6,
                     "traffic_source": "ncu --set full of one k_mul<32> launch (summary committed under profiles/)",
                     "peak_source": "measured in-process: mi_calib_mul32_peak (independent mad.lo.cc/madc.hi.cc "
                                    "chains, the kernel's own instruction mix)",
                     "per_unit": f"{prods32_per_inst} partial products per instance",
                     # operands in and products out once: far below the HBM bound
                     "hbm": hbm_position(4 * in_bytes, ms, measured_peaks().get("hbm_gbs"))},
        "gpu_launches": args.steps,
        "clocks": clk,
        "e2e": e2e,
        "workloads": extra,
    }
    if rank == 0:
        a_cpu, b_cpu = workloads.mul_pairs(n=N_MUL, m=M_MUL)
        out["cpu_baseline"] = dict(cpu_baseline(a_cpu, b_cpu, M_MUL, args.cpu_seconds, "mul", check=got),
                                   unit="products/s")
        # last key of the line, compact: the targets of every benchmark row
        out["targets"] = targets(out, extra)
        print(json.dumps(out))
        if out["cpu_baseline"].get("matches_gpu_first_instances") is False:
            raise SystemExit("bench: GPU products differ from the CPU baseline's")
    ctx.close()


def _r(x, nd=4):
    return None if x is None else round(float(x), nd)


def targets(out: dict, extra: dict) -> dict:
    """One compact object with each benchmark row's position against its
    target: the classical headline against the IMAD ceiling, 4096-bit
    addition against HBM (>= 0.80), the NTT product against the IMAD ceiling,
    the ragged list against the plain per-size-class form (>= 2.0, results
    identical), serving p50/p99 at the fixed offered load, and the
    end-to-end call against the host link."""
    t = {"mul_8192bit": {"frac": _r(out["roofline"]["frac"]), "ms_per_launch": _r(out["ms_per_step"], 5)},
         "e2e": {"frac_link": _r(out["e2e"].get("frac_link")), "link_gbs": _r(out["e2e"].get("link_gbs"), 1)}}
    if "add_4096bit" in extra:
        a = extra["add_4096bit"]
        t["add_4096bit"] = {"frac_hbm": _r(a["roofline"]["frac"]), "ms_per_launch": _r(a["ms_per_launch"], 5),
                            "target": 0.80}
    if "ntt_mul_65536bit" in extra:
        n = extra["ntt_mul_65536bit"]
        t["ntt_mul_65536bit"] = {"frac": _r(n["roofline"]["frac"]), "ms_per_launch": _r(n["ms_per_launch"], 5)}
    if "ragged_200k" in extra:
        g = extra["ragged_200k"]
        t["ragged"] = {"vs_plain": _r(g["ragged_vs_plain"], 3), "ragged_ms": _r(g["ragged_ms"], 4),
                       "results_identical": g["results_identical"], "target": 2.0}
    if "serving" in extra and extra["serving"].get("fixed_load"):
        f = extra["serving"]["fixed_load"]
        t["serving"] = {"offered_req/s": f["offered_req/s"],
                        "batched_p50_p99_ms": [_r(f["batched"]["p50_ms"], 3), _r(f["batched"]["p99_ms"], 3)],
                        "per_request_p50_p99_ms": [_r(f["per_request"]["p50_ms"], 3),
                                                   _r(f["per_request"]["p99_ms"], 3)]}
    if "fused" in extra and "poly_2048limb" in extra["fused"]:
        t["poly_131072bit"] = {"ms_per_launch": _r(extra["fused"]["poly_2048limb"]["ms_per_launch"], 4)}
    return t


def secondary_workloads(args, ctx, dev, stream, world, rank) -> dict:
    """Addition (GB/s, %HBM), NTT multiplication, ragged vs plain, serving and
    the u32-limb variant, each selectable with --sections."""
    res = {}
    sections = set(args.sections.split(","))
    if "add" in sections:
        res["add_4096bit"] = add_section(args, ctx, dev, stream, world, rank)
    if "ntt" in sections:
        res["ntt_mul_65536bit"] = ntt_section(args, ctx, dev, stream, world, rank)
    if "ragged" in sections:
        res["ragged_200k"] = ragged_vs_plain(args, ctx, dev, stream, world, rank)
    if "serving" in sections:
        res["serving"] = serving_sweep(args, ctx, rank)
    if "u32" in sections:
        res["mul_8192bit_u32limbs"] = u32_section(args, ctx, dev, stream, world, rank)
    if "fused" in sections:
        res["fused"] = fused_section(args, ctx, dev, stream, world, rank)
    if "wide" in sections:
        res["wide_add"] = wide_section(args, ctx, dev, stream, world, rank)
    if "sweep" in sections:  # opt-in: not among the defaults
        res["size_sweep"] = size_sweep(args, ctx, dev, stream, world, rank)
    return res


def ref_u32_ops(m32: int) -> float:
    """The reference driver's normalised operation count of one product of
    m32-word operands, 300 m lg m (numAd32OpsOfMultInst, cuda/helper.h:37-43),
    which its Gu32ops/s figures divide by the time."""
    return 300.0 * m32 * (m32.bit_length() - 1)


def size_sweep(args, ctx, dev, stream, world, rank) -> dict:
    """Every size the reference driver sweeps (cuda/main.cu:661-746): operands
    of 16..4096 u32 words (512..131072 bits) with 2^24 words per operand array
    (the instance count shrinks as the size grows); addition in GB/s (3 words
    moved per operand word, the driver's count), the low-half classical
    product (the driver's gpuMultiply semantics) and the NTT product in
    products/s and in the driver's normalised Gu32ops/s.  Two operand sets
    rotate (256 MiB > L2)."""
    import torch

    import workloads

    sp = stream.cuda_stream
    hbm = measured_peaks().get("hbm_gbs")
    total = 1 << 24  # u32 words per operand array
    out = {"config": "operands of 16..4096 u32 words, 2^24 words per operand array, 2 rotating sets",
           "sizes": {}}
    for m32 in (16, 32, 64, 128, 256, 512, 1024, 2048, 4096):
        m = m32 // 2  # u64 limbs
        n = total // m32
        a, b = workloads.mul_pairs(n=n, m=m, seed=workloads.SEED_BASE + 9 + m32, first=instance_range(n, rank)[0])
        with torch.cuda.stream(stream):
            da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(2)]
            db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(2)]
            dr = [torch.empty(2 * a.size, dtype=torch.int64, device=dev) for _ in range(2)]
        torch.cuda.synchronize()
        row = {"instances": n}
        ms = max_over_ranks(world, time_device(lambda i: ctx.add(da[i], db[i], dr[i], n, m, stream=sp), 2, 20, 3,
                                               stream))
        gbs = 3.0 * n * m * 8 / (ms * 1e-3) / 1e9
        row["add"] = {"ms": ms, "GB/s": world * gbs, "frac_hbm": (gbs / hbm) if hbm else None}
        ms = max_over_ranks(world, time_device(lambda i: ctx.mul_lo(da[i], db[i], dr[i], n, m, stream=sp), 2, 10, 3,
                                               stream))
        row["mul_lo"] = {"ms": ms, "products/s": world * n / (ms * 1e-3),
                         "Gu32ops/s": world * n * ref_u32_ops(m32) / (ms * 1e-3) / 1e9}
        ms = max_over_ranks(world, time_device(lambda i: ctx.mul_ntt(da[i], db[i], dr[i], n, m, stream=sp), 2, 10, 3,
                                               stream))
        row["mul_ntt"] = {"ms": ms, "products/s": world * n / (ms * 1e-3),
                          "Gu32ops/s": world * n * ref_u32_ops(m32) / (ms * 1e-3) / 1e9}
        out["sizes"][str(m32 * 32)] = row
        del da, db, dr
        torch.cuda.empty_cache()
    return out


def add_section(args, ctx, dev, stream, world, rank) -> dict:
    import torch

    import workloads

    sp = stream.cuda_stream
    hbm = measured_peaks().get("hbm_gbs")
    a, b = workloads.add_pairs(n=N_ADD, m=M_ADD, first=instance_range(N_ADD, rank)[0])
    set_bytes = 3 * a.nbytes + N_ADD
    sets = max(2, -(-4 * L2_BYTES // set_bytes))
    with torch.cuda.stream(stream):
        da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(sets)]
        db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(sets)]
        dr = [torch.empty(a.size, dtype=torch.int64, device=dev) for _ in range(sets)]
        dc = [torch.empty(N_ADD, dtype=torch.uint8, device=dev) for _ in range(sets)]
    torch.cuda.synchronize()

    def add_step(i):
        ctx.add(da[i], db[i], dr[i], N_ADD, M_ADD, carry=dc[i], stream=sp)

    steps = max(args.steps, 100)
    ms = max_over_ranks(world, time_device(add_step, sets, steps, max(args.warmup, 5), stream))
    algo_bytes = N_ADD * (3 * M_ADD * 8 + 1)
    gbs = algo_bytes / (ms * 1e-3) / 1e9
    out = {
        "config": "plain addition, 65536 pairs x 4096-bit (64 u64 limbs), every 8th pair all-ones + 1; "
                  "sum mod 2^4096 + carry-out byte",
        "ms_per_launch": ms, "GB/s": gbs * world, "instances/s": world * N_ADD / (ms * 1e-3),
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                     "frac": (gbs / hbm) if hbm else None,
                     # one k_add launch under ncu: the two operands read once (67.12 MB), 3.98 MB of the result
                     # written back before the kernel ended (the rest drains from L2 afterwards)
                     "traffic": 67.12e6 + 3.98e6,
                     "traffic_source": "ncu --set full of one k_add launch (summary committed under profiles/)",
                     "per_unit": "1537 B per instance (2 x 512 B read, 512 B + 1 B written)",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm else "absent"},
        "l2": f"{sets} rotating sets of {set_bytes >> 20} MiB",
    }
    del da, db, dr, dc
    torch.cuda.empty_cache()
    return out


def ntt_section(args, ctx, dev, stream, world, rank) -> dict:
    """NTT multiplication: 1024 pairs x 65536-bit, every 16th pair all ones."""
    import torch

    import midint
    import workloads

    sp = stream.cuda_stream
    n_ntt, m_ntt = 1024, 1024
    a, b = workloads.ntt_pairs(n=n_ntt, m=m_ntt, first=instance_range(n_ntt, rank)[0])
    set_bytes = 4 * a.nbytes
    sets = max(2, -(-4 * L2_BYTES // set_bytes))
    with torch.cuda.stream(stream):
        da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(sets)]
        db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(sets)]
        dr = [torch.empty(2 * a.size, dtype=torch.int64, device=dev) for _ in range(sets)]
    torch.cuda.synchronize()
    ms = max_over_ranks(world, time_device(
        lambda i: ctx.mul_ntt(da[i], db[i], dr[i], n_ntt, m_ntt, stream=sp), sets, max(10, args.steps // 2),
        max(3, args.warmup), stream))
    peak = midint.calib_mul32_peak()
    # 5 primes < 2^30: 3 transforms x 1024*11 butterflies (3 multiplies each, Shoup), 2048 pointwise
    # products (4, Montgomery), 2 x 1024 digit conversions (2 x 3) per prime, and Garner's 2048
    # coefficients x (10 x 3 + 10)
    mults = 5 * (3 * 1024 * 11 * 3 + 2048 * 4 + 2 * 1024 * 2 * 3) + 2048 * 40
    achieved = n_ntt * mults / (ms * 1e-3)
    out = {
        "config": "plain NTT multiplication, 1024 pairs x 65536-bit (1024 u64 limbs) -> 131072-bit product, "
                  "every 16th pair all-ones; 5 primes < 2^30, 2048-point transforms, CRT + carry fused",
        "ms_per_launch": ms, "products/s": world * n_ntt / (ms * 1e-3),
        "roofline": {"bound": "int-mul", "achieved": achieved / 1e9, "peak": peak / 1e9,
                     "unit": "G 32x32-bit partial products/s", "frac": achieved / peak,
                     "per_unit": f"{mults} 32x32-bit integer multiplies per instance (five 30-bit primes)",
                     "peak_source": "mi_calib_mul32_peak (measured in-process)",
                     # the canonical schedule (3 primes near 2^62, 64-bit digits, L = 2048: 107520
                     # 64-bit modular multiplies per instance, 12 32x32-bit products each) over the same
                     # time and ceiling: above 1 when the schedule run here needs fewer multiplies
                     "canonical_equivalent_frac": n_ntt * 107520 * 12 / (ms * 1e-3) / peak},
        "l2": f"{sets} rotating sets of {set_bytes >> 20} MiB",
    }
    del da, db, dr
    torch.cuda.empty_cache()
    return out


def u32_section(args, ctx, dev, stream, world, rank) -> dict:
    """The u32-limb variant of the classical multiplication (256 u32 limbs)."""
    import torch

    import workloads

    sp = stream.cuda_stream
    # u32-limb variant of the classical multiplication (same bytes, 256 u32 limbs)
    a, b = workloads.mul_pairs(n=N_MUL, m=M_MUL, first=instance_range(N_MUL, rank)[0])
    set_bytes = 4 * a.nbytes  # a, b and the 2m-limb product
    sets = max(2, -(-4 * L2_BYTES // set_bytes))
    with torch.cuda.stream(stream):
        ha, hb = torch.from_numpy(a.view(np.int64)), torch.from_numpy(b.view(np.int64))
        da = [ha.to(dev) for _ in range(sets)]
        db = [hb.to(dev) for _ in range(sets)]
        dr = [torch.empty(2 * a.size, dtype=torch.int64, device=dev) for _ in range(sets)]
    torch.cuda.synchronize()
    ms = max_over_ranks(world, time_device(
        lambda i: ctx.mul_full(da[i], db[i], dr[i], N_MUL, 2 * M_MUL, limb_bits=32, stream=sp), sets, 20, 3, stream))
    out = {"ms_per_launch": ms, "products/s": world * N_MUL / (ms * 1e-3),
           "l2": f"{sets} rotating sets of {set_bytes >> 20} MiB"}
    del da, db, dr
    torch.cuda.empty_cache()
    return out


def wide_section(args, ctx, dev, stream, world, rank) -> dict:
    """Additions wider than one block: 16 pairs of 2^21 u64 limbs (134 Mbit),
    multi-block tiles chained by decoupled look-back."""
    import torch

    import workloads

    sp = stream.cuda_stream
    hbm = measured_peaks().get("hbm_gbs")
    n, m = 16, 1 << 21
    a, b = workloads.add_pairs(n=n, m=m, seed=workloads.SEED_BASE + 7, worst_every=8, first=instance_range(n, rank)[0])
    with torch.cuda.stream(stream):
        da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(2)]
        db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(2)]
        dr = [torch.empty(a.size, dtype=torch.int64, device=dev) for _ in range(2)]
        dc = [torch.empty(n, dtype=torch.uint8, device=dev) for _ in range(2)]
    torch.cuda.synchronize()
    ms = max_over_ranks(world, time_device(
        lambda i: ctx.add(da[i], db[i], dr[i], n, m, carry=dc[i], stream=sp), 2, max(10, args.steps // 2),
        max(args.warmup, 3), stream))
    status = ctx.device_status()
    gbs = n * (3 * 8 * m + 1) / (ms * 1e-3) / 1e9
    del da, db, dr, dc
    torch.cuda.empty_cache()
    return {"config": f"{n} pairs x {m} u64 limbs ({64 * m >> 20} Mbit), every 8th pair all-ones + 1 "
                      "(carries through every tile); 2 rotating sets of 768 MiB",
            "ms_per_launch": ms, "GB/s": world * gbs, "frac_hbm": (gbs / hbm) if hbm else None,
            "device_status_ok": status == 0}


def fused_section(args, ctx, dev, stream, world, rank) -> dict:
    """The fused composites: 6a + 10b on the addition workload and
    ((a^2 + b)(b^2 + b) + ab) mod 2^8192 on the multiplication workload."""
    import torch

    import workloads

    sp = stream.cuda_stream
    hbm = measured_peaks().get("hbm_gbs")
    a, b = workloads.add_pairs(n=N_ADD, m=M_ADD, first=instance_range(N_ADD, rank)[0])
    sets = max(2, -(-4 * L2_BYTES // (3 * a.nbytes)))
    with torch.cuda.stream(stream):
        da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(sets)]
        db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(sets)]
        dr = [torch.empty(a.size, dtype=torch.int64, device=dev) for _ in range(sets)]
    torch.cuda.synchronize()
    ms6 = max_over_ranks(world, time_device(
        lambda i: ctx.add6(da[i], db[i], dr[i], N_ADD, M_ADD, stream=sp), sets, max(args.steps, 100),
        max(args.warmup, 5), stream))
    gbs = N_ADD * 3 * M_ADD * 8 / (ms6 * 1e-3) / 1e9
    del da, db, dr
    a, b = workloads.mul_pairs(n=N_MUL, m=M_MUL, first=instance_range(N_MUL, rank)[0])
    sets = max(2, -(-4 * L2_BYTES // (3 * a.nbytes)))
    with torch.cuda.stream(stream):
        da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(sets)]
        db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(sets)]
        dr = [torch.empty(a.size, dtype=torch.int64, device=dev) for _ in range(sets)]
    torch.cuda.synchronize()
    msp = max_over_ranks(world, time_device(
        lambda i: ctx.poly(da[i], db[i], dr[i], N_MUL, M_MUL, stream=sp), sets, max(10, args.steps // 2),
        max(args.warmup, 3), stream))
    mslo = max_over_ranks(world, time_device(
        lambda i: ctx.mul_lo(da[i], db[i], dr[i], N_MUL, M_MUL, stream=sp), sets, max(10, args.steps // 2),
        max(args.warmup, 3), stream))
    del da, db, dr
    torch.cuda.empty_cache()
    # the composite at 131072 bits: the transform form (the tuned choice at this
    # size) and the classical form, on the same operands
    import midint

    n2, m2 = 512, 2048
    a, b = workloads.mul_pairs(n=n2, m=m2, seed=workloads.SEED_BASE + 11, first=instance_range(n2, rank)[0])
    sets = max(2, -(-4 * L2_BYTES // (3 * a.nbytes)))
    with torch.cuda.stream(stream):
        da = [torch.from_numpy(a.view(np.int64)).to(dev) for _ in range(sets)]
        db = [torch.from_numpy(b.view(np.int64)).to(dev) for _ in range(sets)]
        dr = [torch.empty(a.size, dtype=torch.int64, device=dev) for _ in range(sets)]
    torch.cuda.synchronize()
    old = ctx.get_tuning(midint.TUNE_POLY_NTT_MIN)
    ms2 = max_over_ranks(world, time_device(
        lambda i: ctx.poly(da[i], db[i], dr[i], n2, m2, stream=sp), sets, max(10, args.steps // 2),
        max(args.warmup, 3), stream))
    out_ntt = dr[0].cpu()
    ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, 2049)
    ms2c = max_over_ranks(world, time_device(
        lambda i: ctx.poly(da[i], db[i], dr[i], n2, m2, stream=sp), sets, 3, 1, stream))
    ctx.set_tuning(midint.TUNE_POLY_NTT_MIN, 0, old)
    same2 = bool(torch.equal(out_ntt, dr[0].cpu()))  # set 0 ran in both forms
    del da, db, dr
    torch.cuda.empty_cache()
    if not same2:
        raise SystemExit("bench: the two forms of the composite differ")
    return {
        "add6": {"config": "6a + 10b mod 2^4096, 65536 pairs x 64 u64 limbs (the addition workload)",
                 "ms_per_launch": ms6, "instances/s": world * N_ADD / (ms6 * 1e-3), "GB/s": world * gbs,
                 "frac_hbm": (gbs / hbm) if hbm else None},
        "poly": {"config": "((a^2 + b)(b^2 + b) + ab) mod 2^8192, 16384 pairs x 128 u64 limbs "
                           "(the multiplication workload); 4 products + 3 sums in one kernel",
                 "ms_per_launch": msp, "instances/s": world * N_MUL / (msp * 1e-3)},
        "mul_lo": {"config": "low 8192 bits of the product, 16384 pairs x 128 u64 limbs (the reference's "
                             "gpuMultiply semantics); anti-diagonals below the middle only",
                   "ms_per_launch": mslo, "products/s": world * N_MUL / (mslo * 1e-3)},
        "poly_2048limb": {"config": f"((a^2 + b)(b^2 + b) + ab) mod 2^131072, {n2} pairs x {m2} u64 limbs; four "
                                    "low-half products on number-theoretic transforms (from the tuned crossover, "
                                    f"{old} limbs), intermediates in shared memory",
                          "ms_per_launch": ms2, "instances/s": world * n2 / (ms2 * 1e-3),
                          "classical_form_ms_per_launch": ms2c, "ntt_vs_classical": ms2c / ms2,
                          "results_identical": same2},
    }


def ragged_vs_plain(args, ctx, dev, stream, world, rank) -> dict:
    """Ragged batch of 200000 mixed ops: the persistent ragged kernels
    (replayed CUDA graph) against the plain per-size-class launches with both
    operands zero-padded to the class.  Both are timed device-resident with
    CUDA events; the two outputs are compared limb for limb."""
    import torch

    import midint
    import workloads
    from plainform import PlainBatch

    ops, pool, out_limbs = ragged_shard(args.ragged_ops, world, rank)
    n = ops.size
    sp = stream.cuda_stream
    with torch.cuda.stream(stream):
        d_ops = torch.from_numpy(ops.view(np.uint8).copy()).to(dev)
        d_in = torch.from_numpy(pool.view(np.int64)).to(dev)
        d_out = torch.empty(out_limbs, dtype=torch.int64, device=dev)
        d_c = torch.empty(n, dtype=torch.uint8, device=dev)
        sb = midint.ragged_scratch_bytes(n)
        scr = torch.empty(sb // 4 + 1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    graph = ctx.ragged_graph(d_ops, n, d_in, d_out, scr, sb, carry=d_c)
    steps = max(5, min(args.steps, 20))
    ms_r = max_over_ranks(world, time_device(lambda i: graph.launch(sp), 1, steps, max(3, args.warmup), stream))
    invalid = midint.ragged_invalid(scr)
    out_r = d_out.cpu().numpy().view(np.uint64).copy()
    carry_r = d_c.cpu().numpy().copy()
    graph.close()

    plain = PlainBatch(ops, pool, device=dev)
    launches = [0]

    def plain_step(i):
        launches[0] = plain.run(ctx, sp)

    ms_p = max_over_ranks(world, time_device(plain_step, 1, steps, max(3, args.warmup), stream))
    out_p, carry_p = plain.results(ops, out_limbs)
    adds = ops["kind"] == 0
    same = bool(np.array_equal(out_r, out_p) and np.array_equal(carry_r[adds], carry_p[adds]))
    la, lb = ops["la"].astype(np.int64), ops["lb"].astype(np.int64)
    muls = ops["kind"] == 1
    del plain, d_ops, d_in, d_out, d_c, scr
    torch.cuda.empty_cache()
    if not same:
        raise SystemExit("bench: ragged and plain-form results differ")
    total = args.ragged_ops * world
    return {
        "config": f"{total} ops, 40% add / 60% mul, operand bits log-uniform in [256, 65536] (4..1024 u64 limbs), "
                  "independent lengths; adds return max(la,lb) limbs + carry, muls la+lb limbs"
                  + (f"; split over {world} ranks by estimated work ({n} ops on rank {rank})" if world > 1 else ""),
        "ragged_ms": ms_r, "ragged_ops/s": total / (ms_r * 1e-3),
        "plain_ms": ms_p, "plain_ops/s": total / (ms_p * 1e-3), "plain_launches": launches[0],
        "ragged_vs_plain": ms_p / ms_r,
        "mul_partial_products": int((la[muls] * lb[muls]).sum() * 4),
        "results_identical": same, "invalid_ops": invalid,
        "ragged_path": "one CUDA graph: classify, scan, scatter, persistent NTT / classical / add kernels",
    }


def ragged_shard(n_per_rank: int, world: int, rank: int):
    """This rank's part of the whole job's ragged list of n_per_rank x world
    ops: the kinds and lengths are drawn for the whole list from one seed
    (the same on every rank), split by estimated work (shard_ragged), and
    the rank's ops are packed with seeded operands of their own.  With one
    rank this is exactly workloads.ragged_ops(n_per_rank)."""
    import workloads

    seed = workloads.SEED_BASE + 3
    total = n_per_rank * world
    rng = np.random.default_rng(seed)
    kind = (rng.random(total) >= 0.4).astype(np.uint32)
    lo, hi = np.log(256), np.log(65536)
    la = np.ceil(np.exp(rng.uniform(lo, hi, total)) / 64).astype(np.uint32)
    lb = np.ceil(np.exp(rng.uniform(lo, hi, total)) / 64).astype(np.uint32)
    if world == 1:
        return workloads.pack_ops(kind, la, lb, seed)
    mine = shard_ragged(ragged_work_estimate(kind, la, lb), world)[rank]
    return workloads.pack_ops(kind[mine], la[mine], lb[mine], rank_seed(seed, rank))


def make_requests(count: int, seed: int):
    """Serving requests: 1..512 ops each, operand bits log-uniform in
    [512, 32768], 50/50 add/mul, seeded limbs."""
    import workloads

    rng = np.random.default_rng(seed)
    reqs = []
    lo, hi = np.log(512), np.log(32768)
    for i in range(count):
        n = int(rng.integers(1, 513))
        kind = rng.integers(0, 2, n).astype(np.uint32)
        la = np.ceil(np.exp(rng.uniform(lo, hi, n)) / 64).astype(np.uint32)
        lb = np.ceil(np.exp(rng.uniform(lo, hi, n)) / 64).astype(np.uint32)
        reqs.append(workloads.pack_ops(kind, la, lb, seed * 7919 + i))
    return reqs


def serve_once(ctx, reqs, rate: float | None, batching: bool, seed: int) -> dict:
    """Submits every request (all at once if rate is None, else at Poisson
    arrival times of that mean rate) and returns throughput and latency."""
    import midint

    outs = [np.zeros(r[2], np.uint64) for r in reqs]
    carries = [np.zeros(r[0].size, np.uint8) for r in reqs]
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, len(reqs)) if rate else np.zeros(len(reqs))
    arrivals = np.cumsum(gaps)
    with midint.Server(ctx, device_bytes=2 << 30, slots=3, batching=batching) as srv:
        tickets = []
        t0 = time.perf_counter()
        for (ops, pool, _), out, c, at in zip(reqs, outs, carries, arrivals):
            while time.perf_counter() - t0 < at:
                pass
            tickets.append(srv.submit(ops, pool, out, c))
        for t in tickets:
            srv.wait(t)
        times = np.array([srv.times(t) for t in tickets], dtype=np.float64)
        batches, _, n_ops = srv.stats()
    lat = (times[:, 2] - times[:, 0]) * 1e-6
    span = (times[:, 2].max() - times[:, 0].min()) * 1e-9
    return {"offered_req/s": rate, "achieved_req/s": len(reqs) / span, "ops/s": n_ops / span,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "batches": batches, "requests": len(reqs)}


def serving_sweep(args, ctx, rank) -> dict:
    """Open-loop Poisson arrivals at fractions of the batched loop's capacity,
    for continuous batching and for the plain per-request launch."""
    reqs = make_requests(400, seed=workloads_seed(rank))
    cap = serve_once(ctx, reqs, None, True, 1)          # closed loop: capacity
    cap_plain = serve_once(ctx, reqs, None, False, 1)
    out = {"config": "400 requests of U[1,512] ops (50/50 add/mul), operand bits log-uniform in [512, 32768]; "
                     "open-loop Poisson arrivals; latency = submit -> results in the caller's host buffers",
           "capacity_batched": cap, "capacity_per_request": cap_plain, "sweep": []}
    for frac in (0.25, 0.5, 0.8):
        rate = frac * cap["achieved_req/s"]
        out["sweep"].append({"load_fraction_of_batched_capacity": frac,
                             "batched": serve_once(ctx, reqs, rate, True, 2),
                             "per_request": serve_once(ctx, reqs, rate, False, 2)})
    # one named offered load, the same in every run
    out["fixed_load"] = {"offered_req/s": SERVE_FIXED_RATE,
                         "batched": serve_once(ctx, reqs, SERVE_FIXED_RATE, True, 3),
                         "per_request": serve_once(ctx, reqs, SERVE_FIXED_RATE, False, 3)}
    return out


def workloads_seed(rank: int) -> int:
    import workloads

    return rank_seed(workloads.SEED_BASE + 4, rank)


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import workloads

    a, b = workloads.mul_pairs(n=N_MUL, m=M_MUL)
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps + args.warmup) * 4)
    for _ in range(min(args.warmup, 3)):
        cpu_baseline(a, b, M_MUL, per_step / 4, "mul")
    vals = []
    cb = None
    t0 = time.perf_counter()
    for _ in range(max(1, min(args.steps, 5))):
        cb = cpu_baseline(a, b, M_MUL, per_step, "mul")
        vals.append(cb["value"])
    wall = time.perf_counter() - t0
    value = statistics.median(vals)
    out = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "products/s",
        "n_gpus": world,
        "steps": len(vals),
        "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / len(vals),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 limbs (GMP mpz_mul)",
        "data": "synthetic: seeded splitmix64 limbs (uniform)",
        "config": {"workload": "plain classical multiplication, 16384 pairs x 8192-bit (128 u64 limbs) -> "
                               "16384-bit full product", "instances_per_gpu": N_MUL, "limbs_u64": M_MUL},
        "cpu_baseline": dict(cb, value=value, unit="products/s"),
        "e2e": {"value": value, "unit": "products/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# --- profiling cases -----------------------------------------------------------

def run_case(args):
    """Profiling cases (--case): one launch of each named kernel family on the
    benchmark's shapes, inputs resident on cuda:0, after --case-warmup untimed
    calls, so that a profiler can capture exactly those launches; or one of
    the timing scans, printed as JSON.  Prints no bench line.

      add     65536 x 64 u64 limbs, carries        (k_add)
      add6    6a + 10b on the same batch            (k_add, 6a+10b variant)
      mul     16384 x 128 u64 limbs, full products  (k_mul)
      mul_lo  the same batch, low halves            (k_mul_lo)
      poly    the same batch                        (k_poly)
      poly2048  512 x 2048 u64 limbs, the composite on transforms (k_poly_ntt)
      ntt     1024 x 1024 u64 limbs                 (k_ntt_mul, 64-bit digits on five primes)
      ntt48   1024 x 768 u64 limbs                  (k_ntt_mul, 48-bit digits on four primes, L = 2048)
      ragged  a mixed ragged list (--case-ragged-ops)  (k_classify, k_scan, k_scatter, k_rg_*)
      wide    16 pairs x 2^21 u64 limbs             (k_add_wide)
      convert the addition batch to big-endian 8-byte words and back (k_export, k_count_words, k_import)
      ragged_bands  the ragged list cut into its additions and its products by
              shorter-operand band, each band timed alone as its own captured
              ragged run (CUDA events over 10 replays after 3)
      ntt_sizes  NTT products at 384/400, 768/800 and 1536/1600 limbs (48-bit
              digits on four primes against 64-bit digits on five at the same
              transform length), ns per product, CUDA events over 10 after 3
      ntt_batches  NTT products of 1024 u64 limbs in batches of 152..2736
              instances, ms per launch, CUDA events over 20 after 3
      wide_variants  16 pairs x 2^21 u64 limbs with no all-ones pair, every
              8th pair all-ones + 1, and every pair all-ones + 1, GB/s
    """
    import torch

    import midint
    import workloads

    dev = torch.device("cuda:0")
    ctx = midint.Context(0)
    sp = torch.cuda.current_stream().cuda_stream

    def dput(x):
        return torch.from_numpy(x.view(np.int64)).to(dev)

    calls = []
    ops = args.case.split(",")
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
    if "poly2048" in ops:
        a2, b2 = workloads.mul_pairs(n=512, m=2048, seed=workloads.SEED_BASE + 11)
        pa, pb = dput(a2), dput(b2)
        pr = torch.empty(a2.size, dtype=torch.int64, device=dev)
        calls.append(lambda: ctx.poly(pa, pb, pr, 512, 2048, stream=sp))
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
        rops, pool, out_limbs = workloads.ragged_ops(n_ops=args.case_ragged_ops)
        d_ops = torch.from_numpy(rops.view(np.uint8).copy()).to(dev)
        d_in = dput(pool)
        d_out = torch.empty(out_limbs, dtype=torch.int64, device=dev)
        d_c = torch.empty(rops.size, dtype=torch.uint8, device=dev)
        sb = midint.ragged_scratch_bytes(rops.size)
        scr = torch.empty(sb // 4 + 1, dtype=torch.int32, device=dev)
        calls.append(lambda: ctx.ragged_run(d_ops, rops.size, d_in, d_out, scr, sb, carry=d_c, stream=sp))
    torch.cuda.synchronize()
    for _ in range(args.case_warmup):
        for c in calls:
            c()
    torch.cuda.synchronize()
    for c in calls:
        c()
    torch.cuda.synchronize()
    if "ragged_bands" in ops:
        print(json.dumps(case_ragged_bands(ctx, dev, sp, args.case_ragged_ops), indent=1))
    if "wide_variants" in ops:
        print(json.dumps(case_wide_variants(ctx, dev, sp), indent=1))
    if "ntt_sizes" in ops:
        print(json.dumps(case_ntt_sizes(ctx, dev, sp), indent=1))
    if "ntt_batches" in ops:
        print(json.dumps(case_ntt_batches(ctx, dev, sp), indent=1))
    ctx.close()
    print("case: ran", ",".join(ops))


def case_ntt_sizes(ctx, dev, sp) -> dict:
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


def case_ntt_batches(ctx, dev, sp) -> dict:
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


def case_wide_variants(ctx, dev, sp) -> dict:
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


def case_ragged_bands(ctx, dev, sp, n_ops: int) -> dict:
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


def main():
    args = parse()
    world, _, _ = dist_env()
    verdict = check_world(args.gpus, world)
    if verdict == "launch":
        # --gpus N without a launcher: start N local ranks under torchrun
        import socket

        s = socket.socket()
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
        s.close()
        raise SystemExit(subprocess.call(launch_command(sys.argv[1:], args.gpus, port)))
    if verdict is not None:
        raise SystemExit(f"bench: {verdict}")
    if args.case:
        run_case(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
