"""Benchmark: reads/s of the SWIFT hot path on GB300.

One step = one pass of the whole pipeline over one batch of reads already
resident on the device: SSAHA seeding of both strands, window construction,
Smith-Waterman (LCS bound with suffix values, traceback of each read's
candidate, exact scores of the pairs the bound keeps, both passes stopped
early), best alignment per read
and the default text records (left on the device).  The one-time index build
is excluded and reported separately; `e2e` repeats the step through
swift_align_into with the reads and the text in pinned host memory.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload scale|batched|long|serving|paired] [--reads N]
                  [--seeder ssaha|lt13] [--format default|sam] [--no-e2e]

Workload "scale" (default): 50 Mbp reference in 24 sequences (log-normal
lengths, 10 % diverged repeat copies), 1,000,000 reads x 100 bp (1 % subs,
0.1 % indels, 5 % random reads); seeded synthetic data.  With N GPUs each rank
aligns its own 1M reads (weak scaling; no collective on the data path).

--impl reference times the reference algorithm's CPU implementation (the
oracle port, multithreaded over all host cores) on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "reads/s (SSAHA seeding + Smith-Waterman + best per read + records), bit-exact"
METRIC_LT13 = ("reads/s (lt13 seed-and-extend seeding + Smith-Waterman + best per read + "
               "records), bit-exact")


def metric_for(args):
    return METRIC_LT13 if args.seeder == "lt13" else METRIC
# The candidates' trace pass (up to its early stop), per pair: algorithmic
# bytes 112 B query + 304 B window read and 8 B first maximum, plus the
# direction words written for the steps it ran (8 lanes x 2 words x 4 B per
# step for two pairs at 100 bp: 32 B per step and pair, 100 cells a step, so
# 0.32 B per cell computed).  DRAM bytes per cell computed, read + written,
# from one ncu capture of the candidates' launch (210,162 pairs of the scale
# workload with 200 K reads, 4.44 G cells computed: 161.0 MB read, 1416.5 MB
# written).
TRACE_DRAM_BYTES_PER_CELL = (161.0e6 + 1416.5e6) / 4.437e9
TRACE_ALGO_BYTES_PER_PAIR = 112 + 304 + 8
TRACE_DIR_BYTES_PER_CELL = 8 * 2 * 4 / 2 / 100
# ALU-pipe instructions the trace pass issues per 2 cells computed (per
# lane), from the same capture: 612.4 M warp instructions on the ALU pipe
# (1193.2 M in all) for 4.44 G cells, the early-stop tests included.
TRACE_ALU_PER_2_CELLS = 8.83
TRACE_NOTE = ("the trace formulation issues about 8.8 ALU-pipe instructions per 2 cells (the "
              "substitution permute, two DPX max ops, three masks, the first-maximum add-max, "
              "the early-stop tests) and 17.2 instructions in all, so about 0.11 is its ceiling")
SCORE_NOTE = ("the exact formulation issues about 6.5 ALU instructions per 2 cells, so about "
              "0.15 is its ceiling")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="scale",
                    choices=["scale", "small", "batched", "serving", "long", "paired"])
    ap.add_argument("--format", default="default", choices=["default", "sam"],
                    help="output records: the default text or SAM (-f 1)")
    ap.add_argument("--reads", type=int, default=None)
    ap.add_argument("--read-len", type=int, default=100,
                    help="scale workload: read length (reads past 199 bases set max_read_len 300)")
    ap.add_argument("--ref-mbp", type=int, default=50,
                    help="scale workload: reference size in Mbp (24 sequences)")
    ap.add_argument("--cpu-sample", type=int, default=20000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--serve-workers", type=int, default=4,
                    help="serving: concurrent wave pipelines")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the short runs of the batched, long-region and serving "
                         "configurations that the default line carries")
    ap.add_argument("--seeder", default="ssaha", choices=["ssaha", "lt13"],
                    help="Phase 1: SSAHA seeding (searchQueries3) or lt13 seed-and-extend "
                         "(search2Queries, the reference CLI's GPU default)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float) -> float:
    """The largest x over the ranks of the process group (a job takes as long
    as its slowest replica): a device tensor on NCCL, a host one on gloo."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: int, world: int, steps: int, seconds: float) -> float:
    """Whole-job units per second: every replica processes its own units
    (weak scaling), timed by the slowest one."""
    return units_per_rank * world * steps / seconds


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.file:
            return None
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def make_workload(args, rank):
    from swift_gb300 import synth
    if args.workload == "small":
        names, seqs = synth.make_reference(1_000_000, 1, seed=0)
        n = args.reads or 10_000
        rn, rs, orig = synth.make_reads(seqs, n, 100, 0.01, 0.001, 0.0, seed=1 + rank)
        desc = "small: 1 Mbp / 1 seq, %d x 100 bp reads" % n
    else:
        names, seqs = synth.make_reference(args.ref_mbp * 1_000_000, 24, sigma=0.8,
                                           repeat_frac=0.10, n_units=500, unit_len=300,
                                           divergence=0.03, seed=0)
        n = args.reads or 1_000_000
        rn, rs, orig = synth.make_reads(seqs, n, args.read_len, 0.01, 0.001, 0.05, seed=1 + rank)
        desc = ("scale: %d Mbp / 24 seqs (log-normal sigma 0.8, 10%% repeats of 500 x 300 bp "
                "units at 3%% divergence), %d x %d bp reads (1%% subs, 0.1%% indels, 5%% random)"
                % (args.ref_mbp, n, args.read_len))
    wl = {"seqs": seqs, "reads": rs, "origins": orig}
    return synth.fasta_bytes(names, seqs), synth.reads_fasta(rn, rs), n, desc, wl


def sample_reads(reads: bytes, n: int) -> bytes:
    lines = reads.split(b"\n", 2 * n)
    return b"\n".join(lines[: 2 * n]) + b"\n"


def cpu_reference(ref: bytes, reads: bytes, n_sample: int, steps: int, warmup: int,
                  seeder: int = 0, device_mem: int = 0, max_read_len: int = 0,
                  out_format: int = 0):
    """The reference algorithm on the host cores (oracle port): reads/s,
    threads, seconds, and the last run's output (for the parity check)."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    sess = O.Session(ref, O.default_params(threads=threads, seeder=seeder,
                                           device_mem=device_mem, max_read_len=max_read_len,
                                           out_format=out_format))
    sample = sample_reads(reads, n_sample)
    for _ in range(warmup):
        sess.align(sample)
    t0 = time.perf_counter()
    out = b""
    for _ in range(steps):
        out = sess.align(sample)
    dt = time.perf_counter() - t0
    return n_sample * steps / dt, threads, dt, out


def cpu_model() -> str:
    """The host CPU's model name (/proc/cpuinfo, else lscpu)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        outp = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in outp.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.machine()


def workload_pairs(seqs, reads_list, origins, n: int, seed: int = 7):
    """The scale workload's Smith-Waterman pairs in the alignSequences layout:
    each read's first n against the 300-base window the reference builds
    around its origin (refPos - 100; a random position for random reads)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    Q, R = 100, 300
    q = np.zeros((n, Q + 1), np.uint8)
    w = np.zeros((n, R + 1), np.uint8)
    for i in range(n):
        q[i, :Q] = np.frombuffer(reads_list[i][:Q], np.uint8)
        sid, pos = origins[i]
        if sid < 0:
            sid = int(rng.integers(0, len(seqs)))
            pos = int(rng.integers(0, max(1, len(seqs[sid]) - R)))
        a = max(0, pos - 100)
        win = np.frombuffer(seqs[sid][a:a + R], np.uint8)
        w[i, :len(win)] = win
    return q, w, Q, R


def cpu_sw_baseline(q, w, Q, R, n):
    """The port's Smith-Waterman (the reference kernel's semantics) over n
    pairs on every host core: GCUPS, threads, seconds."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    qb, wb = q[:n].tobytes(), w[:n].tobytes()
    O.sw_batch(qb, Q, wb, R, min(n, 256), threads=threads)  # warm-up
    t0 = time.perf_counter()
    O.sw_batch(qb, Q, wb, R, n, threads=threads)
    dt = time.perf_counter() - t0
    return n * Q * R / dt / 1e9, threads, dt


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) of this machine's GPUs, or the
    recipe's fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def pairs_run(ctx, kind: str, n_reads: int, steps: int, warmup: int, seed: int, seqs=None,
              plain: bool = True):
    """Phase 2 alone on explicit pairs through swift_sw_pairs, inputs resident
    on the device, coordinates only.  kind "batched": reads 36-250 bp x 1-64
    regions (BASELINE config 2); "long": queries 1-4 kbp x one region of
    2-8 kbp (config 3).  Returns the measured figures: GCUPS of the
    shape-sorted batched mode and, for "batched", of the plain mode (every
    pair padded to the largest shape, one launch) on a tenth of the pairs."""
    import ctypes as C
    import numpy as np
    import torch
    import swift_gb300 as sg
    from swift_gb300 import synth
    if kind == "long":
        ref, reads, qo, ql, ro, rl = synth.long_workload(n_reads, seed=seed)
    else:
        ref, reads, qo, ql, ro, rl = synth.pairs_workload(n_reads, seed=seed, ref=seqs)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    d = dict(q=dev(np.frombuffer(reads, np.uint8)), r=dev(np.frombuffer(ref, np.uint8)),
             qo=dev(qo), ql=dev(ql), ro=dev(ro), rl=dev(rl))
    n = len(ql)
    outs = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(4)]
    torch.cuda.synchronize()

    def run(count, mode):
        st = sg.PairsStats()
        rc = sg.lib().swift_sw_pairs(
            ctx._h, d["q"].data_ptr(), d["qo"].data_ptr(), d["ql"].data_ptr(), d["r"].data_ptr(),
            d["ro"].data_ptr(), d["rl"].data_ptr(), count, 2, -1, -10, -1,
            *(o.data_ptr() for o in outs), None, None, 0, mode, C.byref(st))
        if rc != 0:
            raise sg.SwiftError(rc, sg.lib().swift_last_error(ctx._h).decode())
        return st.as_dict()

    for _ in range(max(warmup, 3)):
        run(n, 0)
    sts = [run(n, 0) for _ in range(steps)]
    ms = statistics.median(s["ms"] for s in sts)
    cells = sts[-1]["cells"]
    res = {"pairs": n, "cells": cells, "ms": ms, "gcups": cells / (ms * 1e-3) / 1e9,
           "segments": sts[-1]["segments"], "generic_pairs": sts[-1]["generic_pairs"],
           "launches": int(sum(s["launches"] for s in sts)), "steps": steps,
           "warmup": max(warmup, 3)}
    if kind != "long" and plain:  # plain mode takes pairs up to 256 x 1024 only
        n_plain = max(1, n // 10)
        run(n_plain, 1)
        sp = [run(n_plain, 1) for _ in range(max(1, min(steps, 2)))]
        ms_p = statistics.median(s["ms"] for s in sp)
        res["plain"] = {"gcups": sp[-1]["cells"] / (ms_p * 1e-3) / 1e9, "pairs": n_plain,
                        "ms": ms_p,
                        "note": "every pair padded to the largest shape, one int32 launch"}
        res["batched_vs_plain"] = res["gcups"] / res["plain"]["gcups"]
    res["workload"] = (("long: %d queries L ~ U[1000,4000] (3%% subs, 0.5%% indels) x one region "
                        "U[max(2000, L+200), 8000] on a 100 Mbp uniform reference" % n_reads)
                       if kind == "long" else
                       ("batched: %d reads L ~ U[36,250] x U{1..64} regions (true + decoys, "
                        "64 bp flanks) on the 50 Mbp reference" % n_reads))
    return res


def bench_batched(args, rank, world, local):
    """Phase 2 alone on read x region pairs of varying lengths (config 2) or
    long pairs (config 3), both bit-exact; see pairs_run."""
    import torch
    import swift_gb300 as sg
    from swift_gb300 import build as b
    device = local
    torch.cuda.set_device(device)
    b.build()
    long = args.workload == "long"
    stream = torch.cuda.Stream(device)
    torch.cuda.set_stream(stream)
    ctx = sg.Context(device, stream.cuda_stream)
    n_reads = args.reads or (20_000 if long else 1_000_000)
    with ClockSampler(device) as clk:
        res = pairs_run(ctx, "long" if long else "batched", n_reads, args.steps, args.warmup,
                        seed=1 + rank)
    if rank == 0:
        print(json.dumps({
            "metric": ("SW GCUPS on long query x region pairs, bit-exact" if long else
                       "SW GCUPS on read x region pairs of varying length (batched), bit-exact"),
            "value": res["gcups"], "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
            "warmup": res["warmup"], "ms_per_step": res["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32" if long else "int16x2",
            "data": "synthetic",
            "config": {"workload": res["workload"], "pairs": res["pairs"], "cells": res["cells"],
                       "segments": res["segments"], "generic_pairs": res["generic_pairs"]},
            "plain": res.get("plain"),
            "batched_vs_plain": res.get("batched_vs_plain"),
            "gpu_launches": res["launches"],
            "clocks": clk.summary(),
        }))
    return 0


SERVE_MAX_READ = 300  # read lengths of the serving workload: U[50, SERVE_MAX_READ]


def serving_pool(seqs, pool_size: int, seed: int, max_len: int = SERVE_MAX_READ):
    """Requests of the serving workload: log-uniform sizes in [1, 10000]
    reads, each request's reads of one length U[50, max_len] with the
    config-0 error model (5 % random reads)."""
    import numpy as np
    from swift_gb300 import synth
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(0, np.log(10001), pool_size))).astype(int).clip(1, 10000)
    # reads drawn once at the longest length, each request cut to its own
    _, rs_all, _ = synth.make_reads(seqs, int(sizes.sum()), max_len, 0.01, 0.001, 0.05,
                                    seed=seed + 1000)
    pool, at = [], 0
    for t, n in enumerate(sizes):
        L = int(rng.integers(50, max_len + 1))
        rs = [r[:L] for r in rs_all[at:at + int(n)]]
        at += int(n)
        pool.append((int(n), synth.reads_fasta([f"s{t}_{i}" for i in range(int(n))], rs)))
    return pool


def serving_run(idx, device, seqs, pool_size=120, per_load=200, loads=(0.8,), seed=3,
                workers=4):
    """Serving on a resident index: the saturation throughput (every request
    of the pool queued at once), then Poisson arrivals at fractions of it,
    with per-request latency from submission to result (p50 / p99)."""
    import numpy as np
    import swift_gb300 as sg
    rng = np.random.default_rng(seed + 7)
    pool = serving_pool(seqs, pool_size, seed)
    srv = sg.Server(idx, device=device, workers=workers,
                    params=sg.default_params(max_read_len=SERVE_MAX_READ))
    try:
        for n, r in pool[:8]:  # warm-up
            srv.wait(srv.submit(r))
        t0 = time.perf_counter()
        tickets = [srv.submit(r) for _, r in pool]
        sat_st = [srv.wait(t)[1] for t in tickets]
        sat_s = time.perf_counter() - t0
        sat_waves = [x["wave_requests"] for x in sat_st]
        total_reads = sum(n for n, _ in pool)
        sat_rps = total_reads / sat_s
        mean_reads = total_reads / len(pool)
        out = []
        for frac in loads:
            rate = frac * sat_rps / mean_reads  # requests per second
            gaps = rng.exponential(1.0 / rate, per_load)
            picks = rng.integers(0, len(pool), per_load)
            lat, done_reads = [], 0
            start = time.perf_counter()
            due = start
            tks = []
            for g, k in zip(gaps, picks):
                due += g
                now = time.perf_counter()
                if due > now:
                    time.sleep(due - now)
                tks.append((srv.submit(pool[k][1]), pool[k][0]))
            waves = []
            for t, n in tks:
                _, st = srv.wait(t)
                lat.append(st["total_ms"])
                waves.append(st["wave_requests"])
                done_reads += n
            el = time.perf_counter() - start
            out.append({"offered_fraction": frac, "offered_reads_per_s": frac * sat_rps,
                        "achieved_reads_per_s": done_reads / el, "requests": per_load,
                        "p50_ms": float(np.percentile(lat, 50)),
                        "p99_ms": float(np.percentile(lat, 99)),
                        "mean_requests_per_wave": float(np.mean(waves))})
    finally:
        srv.close()
    return {"saturation_reads_per_s": sat_rps, "saturation_s": sat_s, "pool_requests": pool_size,
            "saturation_mean_requests_per_wave": float(np.mean(sat_waves)),
            "saturation_host_ms": {  # per request: its parse, its wave's pipeline call
                "parse_median": float(np.median([x["parse_ms"] for x in sat_st])),
                "wave_median": float(np.median([x["wave_ms"] for x in sat_st])),
                "device_median": float(np.median([x["device_ms"] for x in sat_st]))},
            "mean_reads_per_request": mean_reads, "workers": workers,
            "read_length": "U[50, %d] per request" % SERVE_MAX_READ, "latency": out}


def bench_serving(args, rank, world, local):
    """Serving (config 4): a 200 Mbp reference (24 sequences) resident;
    requests of log-uniform size in [1, 10000] reads; see serving_run."""
    import swift_gb300 as sg
    from swift_gb300 import build as b, synth
    import torch
    torch.cuda.set_device(local)
    b.build()
    names, seqs = synth.make_reference(200_000_000, 24, sigma=0.8, repeat_frac=0.10,
                                       n_units=500, unit_len=300, divergence=0.03, seed=0)
    ctx = sg.Context(local)
    idx = ctx.index(synth.fasta_bytes(names, seqs))
    with ClockSampler(local) as clk:
        res = serving_run(idx, local, seqs, pool_size=240, per_load=500,
                          loads=(0.3, 0.6, 0.8, 0.9), seed=3 + rank, workers=args.serve_workers)
    if rank == 0:
        print(json.dumps({
            "metric": "serving reads/s at saturation; p50/p99 request latency under Poisson load",
            "value": res["saturation_reads_per_s"], "unit": "reads/s", "n_gpus": world,
            "steps": len(res["latency"]), "warmup": 8, "ms_per_step": res["saturation_s"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16x2",
            "data": "synthetic",
            "config": {"workload": "serving: 200 Mbp / 24 seqs resident; %d-request pool, sizes "
                       "log-uniform [1, 10000] reads (mean %.0f), read length %s"
                       % (res["pool_requests"], res["mean_reads_per_request"],
                          res["read_length"])},
            "latency": res["latency"], "workers": res["workers"],
            "saturation_mean_requests_per_wave": res["saturation_mean_requests_per_wave"],
            "saturation_host_ms": res["saturation_host_ms"], "clocks": clk.summary(),
        }))
    return 0


def bench_paired(args, rank, world, local):
    """Paired-end alignment (-q / -q2) end to end through swift_align_paired_into
    (reads files in pinned host memory in, text out into a pinned host
    buffer): the scale reference, 500 K read pairs, fragments U[200, 500],
    100 bp mates, 1 % substitutions."""
    import torch
    import swift_gb300 as sg
    from swift_gb300 import build as b
    from swift_gb300 import synth
    from oracle import oracle as O
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    n = args.reads or 500_000
    names, seqs = synth.make_reference(50_000_000, 24, sigma=0.8, repeat_frac=0.10,
                                       n_units=500, unit_len=300, divergence=0.03, seed=0)
    ref = synth.fasta_bytes(names, seqs)
    r1, r2 = synth.paired_reads(seqs, n, 100, (200, 500), 0.01, seed=1 + rank)
    desc = ("paired: scale reference (50 Mbp / 24 seqs), %d read pairs, 100 bp mates, "
            "fragments U[200,500], 1%% substitutions" % n)
    metric = ("read pairs/s (paired end: lookupTable2 seeding + Smith-Waterman + mate pairing "
              "+ records), bit-exact")
    fmt = 1 if args.format == "sam" else 0
    if args.impl == "reference":
        if rank != 0:
            return 0
        k = min(args.cpu_sample, n, 5000)
        s1 = sample_reads(r1, k)
        s2 = sample_reads(r2, k)
        p = O.default_params(out_format=fmt)
        t0 = time.perf_counter()
        steps = max(args.steps, 1)
        for _ in range(steps):
            O.align_paired(ref, s1, s2, p)
        dt = time.perf_counter() - t0
        v = k * steps / dt
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": v, "unit": "read pairs/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": 0, "ms_per_step": dt * 1e3 / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "config": {"workload": desc, "sample_pairs_per_step": k},
            "cpu_baseline": {"value": v, "unit": "read pairs/s", "cores": 1, "kind": "port",
                             "sample": f"{k} read pairs per step (index built inside)"},
            "e2e": {"value": v, "unit": "read pairs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}))
        return 0
    torch.cuda.set_device(local)
    b.build()
    ctx = sg.Context(local)
    idx = ctx.index(ref)
    p = sg.default_params(out_format=fmt)
    text = ctx.align_paired(idx, r1, r2, p)
    pin = []
    for r in (r1, r2):
        t = torch.empty(len(r), dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = memoryview(r)
        pin.append(t)
    cap = int(len(text) * 1.1) + (1 << 20)
    out = torch.empty(cap, dtype=torch.uint8, pin_memory=True)

    def call():
        return ctx.align_paired_into(idx, pin[0].data_ptr(), len(r1), pin[1].data_ptr(), len(r2),
                                     out.data_ptr(), cap, p)
    for _ in range(max(args.warmup, 3)):
        out_n, st = call()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    stats = []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            out_n, st = call()
            stats.append(st)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    if world > 1:
        dt = max_over_ranks(dt)
        torch.distributed.barrier()
    if rank != 0:
        return 0
    value = job_throughput(n, world, args.steps, dt)
    dev_ms = statistics.median(s["total_ms"] for s in stats)
    k = min(args.cpu_sample, n, 2000)
    t0 = time.perf_counter()
    O.align_paired(ref, sample_reads(r1, k), sample_reads(r2, k), O.default_params(out_format=fmt))
    cdt = time.perf_counter() - t0
    line = {
        "metric": metric, "value": value, "unit": "read pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16x2",
        "data": "synthetic",
        "config": {"workload": desc, "format": args.format,
                   "records_per_step": stats[-1]["records"],
                   "printed_per_step": stats[-1]["printed"]},
        "phase_ms": {kk: statistics.median(s[kk] for s in stats)
                     for kk in ("seed_ms", "pairs_ms", "sw_ms", "select_ms", "format_ms",
                                "total_ms")},
        "device_pairs_per_s": n / (dev_ms * 1e-3),
        "cpu_baseline": {"value": k / cdt, "unit": "read pairs/s", "cores": 1, "kind": "port",
                         "sample": f"{k} read pairs, index built inside"},
        "e2e": {"value": value, "unit": "read pairs/s", "h2d_bytes_per_step": len(r1) + len(r2),
                "d2h_bytes_per_step": out_n},
        "gpu_launches": int(sum(s["launches"] for s in stats)),
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return 0
        ref, reads, n, desc, _ = make_workload(args, 0)
        steps, warm = max(args.steps, 1), max(args.warmup, 0)
        n_sample = min(args.cpu_sample, n)
        rps, threads, dt, _ = cpu_reference(ref, reads, n_sample, steps, min(warm, 1),
                                            1 if args.seeder == "lt13" else 0,
                                            max_read_len=300 if args.read_len > 199 else 0,
                                            out_format=1 if args.format == "sam" else 0)
        line = {
            "impl": "reference", "metric": metric_for(args), "value": rps, "unit": "reads/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": dt * 1e3 / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": desc, "seeder": args.seeder, "format": args.format,
                       "sample_reads_per_step": n_sample},
            "cpu_baseline": {"value": rps, "unit": "reads/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"{n_sample} reads of the workload per step"},
            "e2e": {"value": rps, "unit": "reads/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return 0

    if args.workload in ("batched", "long"):
        return bench_batched(args, rank, world, local)
    if args.workload == "paired":
        return bench_paired(args, rank, world, local)
    if args.workload == "serving":
        return bench_serving(args, rank, world, local)
    import torch
    import swift_gb300 as sg
    from swift_gb300 import build as b
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local
    torch.cuda.set_device(device)
    b.build()
    ref, reads, n, desc, wl = make_workload(args, rank)
    # a dedicated (non-default) stream shared by the library and the events
    stream = torch.cuda.Stream(device)
    torch.cuda.set_stream(stream)
    ctx = sg.Context(device, stream.cuda_stream)
    t0 = time.perf_counter()
    idx = ctx.index(ref)
    torch.cuda.synchronize()
    index_s = time.perf_counter() - t0
    rd = ctx.reads(reads)
    peak_cells = ctx.peak_dpx_cells_per_s()
    seeder = 1 if args.seeder == "lt13" else 0
    max_read = 300 if args.read_len > 199 else 0
    params = sg.default_params(seeder=seeder, out_format=1 if args.format == "sam" else 0,
                               max_read_len=max_read)
    # warm start: the index written to a file and read back (its load time)
    index_load_s = None
    try:
        import tempfile
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "ref.swidx")
            idx.save(path)
            t0 = time.perf_counter()
            idx2 = sg.Index.load(ctx, path)
            torch.cuda.synchronize()
            index_load_s = time.perf_counter() - t0
            idx2.close()
    except Exception:
        pass
    stats = []
    for _ in range(max(args.warmup, 3)):
        out_n, st = ctx.align_resident(idx, rd, params)
    # timed region: K steps bracketed by barrier + synchronize
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(device) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            out_n, st = ctx.align_resident(idx, rd, params)
            stats.append(st)
        e1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1)
    if world > 1:
        ms = max_over_ranks(ms)
    ms_step = ms / args.steps
    value = job_throughput(n, world, args.steps, ms * 1e-3)
    # Phase 2 = Smith-Waterman passes + selection + traceback phase
    p2_ms = statistics.median(s["sw_ms"] + s["select_ms"] + s["traceback_ms"] for s in stats)
    cells = stats[-1]["cells"]
    gcups = cells / (p2_ms * 1e-3) / 1e9
    gcups_computed = stats[-1]["sw_cells_computed"] / (p2_ms * 1e-3) / 1e9
    # end to end through the C ABI: host reads (pinned) in, host text out
    e2e = None
    if not args.no_e2e:
        pinned = torch.empty(len(reads), dtype=torch.uint8, pin_memory=True)
        pinned.numpy()[:] = memoryview(reads)
        cap = int(out_n * 1.1) + (1 << 20)
        out_pinned = torch.empty(cap, dtype=torch.uint8, pin_memory=True)
        for _ in range(2):
            ctx.align_into(idx, pinned.data_ptr(), len(reads), out_pinned.data_ptr(), cap, params)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        out_bytes = 0
        host = []
        for _ in range(args.steps):
            out_bytes, est = ctx.align_into(idx, pinned.data_ptr(), len(reads),
                                            out_pinned.data_ptr(), cap, params)
            host.append(est)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e2e_s = time.perf_counter() - t0
        if world > 1:
            e2e_s = max_over_ranks(e2e_s)
        e2e = {"value": job_throughput(n, world, args.steps, e2e_s), "unit": "reads/s",
               "h2d_bytes_per_step": len(reads), "d2h_bytes_per_step": out_bytes,
               "ms_per_step": e2e_s * 1e3 / args.steps,
               "host_ms": {k: statistics.median(h[k] for h in host)
                           for k in ("host_parse_ms", "h2d_ms", "d2h_ms", "total_ms")}}
    if rank != 0:
        return 0
    cpu = parity = cpu_sw = None
    k_cpu = min(args.cpu_sample, n)
    model = cpu_model()
    try:
        rps, threads, dt, cpu_out = cpu_reference(ref, reads, k_cpu, 1, 0, seeder,
                                                  device_mem=ctx.info()["total_mem"],
                                                  max_read_len=max_read,
                                                  out_format=params.out_format)
        cpu = {"value": rps, "unit": "reads/s", "cores": threads, "kind": "port",
               "cpu_model": model,
               "sample": f"{k_cpu} reads of the workload, index prebuilt"}
        # the same sample through the GPU path, byte for byte against the
        # oracle's output of the CPU baseline run
        gpu_out = ctx.align(idx, sample_reads(reads, k_cpu), params)
        parity = {"reads": k_cpu, "bytes": len(cpu_out), "bytes_equal": gpu_out == cpu_out,
                  "checked_against": "oracle (CPU restatement of the reference path)"}
    except Exception as ex:  # the baseline must not break the GPU line
        cpu = {"value": None, "unit": "reads/s", "cores": os.cpu_count(), "kind": "port",
               "cpu_model": model, "sample": f"failed: {ex}"}
    try:
        # Smith-Waterman alone: the port's routine on every host core against
        # swift_sw_batch (the alignSequences equivalent) on the same pairs
        n_sw = min(n, 40_000)
        q, w, Q, R = workload_pairs(wl["seqs"], wl["reads"], wl["origins"], n_sw)
        gc, threads, dt = cpu_sw_baseline(q, w, Q, R, n_sw)
        ctx.sw_batch_arrays(q, w, Q, R)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.sw_batch_arrays(q, w, Q, R)
        gdt = time.perf_counter() - t0
        cpu_sw = {"gcups": gc, "pairs": n_sw, "shape": f"{Q} x {R}", "cores": threads,
                  "kind": "port", "cpu_model": model, "seconds": dt,
                  "gpu_sw_batch_gcups": n_sw * Q * R / gdt / 1e9,
                  "gpu_note": "swift_sw_batch on the same pairs, host buffers in and out "
                              "(copies included), every cell computed"}
    except Exception as ex:
        cpu_sw = {"gcups": None, "note": f"failed: {ex}"}
    # the dominant kernel alone, CUDA events on the library's stream: the
    # trace pass of the candidates (up to their early stop), or of every pair
    # over whole windows for SAM
    last = stats[-1]
    tr_ms = statistics.median(s["trace_ms"] for s in stats)
    fp_ms = statistics.median(s["first_pass_ms"] for s in stats)
    peak = peak_cells / 1e9
    fast_pairs = last["records"] - last["sw_generic_pairs"]
    traced = last["traced_pairs"] - last["retraced_pairs"]
    if tr_ms > 0:
        rf_kernel = ("sw_packed_kernel trace pass (%s)"
                     % ("every packed pair, SAM output, whole windows" if args.format == "sam"
                        else "each read's candidate pair, up to the early stop; cells counted "
                             "over the columns every lane of a warp finished"))
        rf_ms, rf_cells = tr_ms, last["trace_cells"]
        rf_traffic = TRACE_DRAM_BYTES_PER_CELL * rf_cells
        rf_algo = TRACE_ALGO_BYTES_PER_PAIR * traced + TRACE_DIR_BYTES_PER_CELL * rf_cells
        rf_note = TRACE_NOTE
    else:
        rf_kernel, rf_ms, rf_cells = "sw_packed_kernel score pass", fp_ms, last["first_pass_cells"]
        rf_traffic, rf_algo, rf_note = None, (112 + 304 + 4) * fast_pairs, SCORE_NOTE
    achieved = rf_cells / (rf_ms * 1e-3) / 1e9 if rf_ms > 0 else None
    # seeding against HBM: the survey's sector-model bytes (counted on the
    # device per strand) over the warp kernels' CUDA-event time
    seed_rf = None
    if args.seeder == "ssaha" and last["seed_kernel_ms"] > 0:
        sk_ms = statistics.median(s["seed_kernel_ms"] for s in stats)
        hbm, hbm_src = hbm_peak()
        ach = last["seed_model_bytes"] / (sk_ms * 1e-3) / 1e9
        seed_rf = {"bound": "hbm", "kernel": "seed_fast_kernel + seed_hash_kernel + seed_overflow_kernel",
                   "model_bytes": last["seed_model_bytes"], "kernel_ms": sk_ms,
                   "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                   "peak_source": hbm_src + " HBM copy bandwidth",
                   "model": "per read strand ceil(L/4) + 32 B per k-mer lookup + "
                            "32 * ceil(5 n / 32) B per occupied bucket of n postings + 12 B "
                            "per hit out; on the 50 Mbp reference the bucket directory and "
                            "postings (about 70 MB) stay resident in L2"}
    # short seeded runs of BASELINE configs 2 and 3 (config 4, serving, below)
    configs = None
    if not args.no_configs and args.workload == "scale" and args.format == "default":
        configs = {}
        for name, kw in (("batched", dict(n_reads=100_000, seed=11, seqs=wl["seqs"])),
                         ("long", dict(n_reads=2_000, seed=12))):
            try:
                with ClockSampler(device) as cclk:
                    configs[name] = pairs_run(ctx, name, steps=5, warmup=3, **kw)
                configs[name]["clocks"] = cclk.summary()
            except Exception as ex:
                configs[name] = {"error": str(ex)}
        try:
            from swift_gb300 import synth
            s_names, s_seqs = synth.make_reference(200_000_000, 24, sigma=0.8, repeat_frac=0.10,
                                                   n_units=500, unit_len=300, divergence=0.03,
                                                   seed=0)
            s_idx = ctx.index(synth.fasta_bytes(s_names, s_seqs))
            with ClockSampler(device) as cclk:
                configs["serving"] = serving_run(s_idx, device, s_seqs,
                                                 workers=args.serve_workers)
            configs["serving"]["clocks"] = cclk.summary()
            configs["serving"]["workload"] = ("serving: 200 Mbp / 24 seqs resident; request "
                                              "sizes log-uniform [1, 10000] reads")
            s_idx.close()
        except Exception as ex:
            configs["serving"] = {"error": str(ex)}
    line = {
        "metric": metric_for(args), "value": value, "unit": "reads/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int16x2" if stats[-1]["sw_generic_pairs"] < stats[-1]["records"] else "int32",
        "data": "synthetic",
        "config": {"workload": desc, "seeder": args.seeder, "format": args.format,
                   "l2": "inputs larger than L2 (reads %.0f MB, index %.0f MB)"
                   % (len(reads) / 1e6, (2 * 4 ** 12 * 4 + 8 * idx.info()["total"]) / 1e6),
                   "records_per_step": stats[-1]["records"],
                   "printed_per_step": stats[-1]["printed"],
                   "generic_pairs_per_step": stats[-1]["sw_generic_pairs"],
                   "traced_pairs_per_step": stats[-1]["traced_pairs"],
                   "retraced_pairs_per_step": stats[-1]["retraced_pairs"],
                   "bound_pruned_pairs_per_step": stats[-1]["bound_pruned"],
                   "index_build_s": index_s, "index_load_s": index_load_s},
        "sw_gcups": gcups,
        "sw_gcups_kind": ("effective: all Q x R cells of every record / Phase-2 device time "
                          "(Smith-Waterman passes + selection + traceback phase, %.2f ms); the "
                          "bounds rule most cells out without computing them" % p2_ms),
        "sw_gcups_computed": gcups_computed,
        "sw_gcups_computed_kind": ("DP cells the kernels computed (trace and exact score "
                                   "passes up to their early stop, generic) / the same time"),
        "parity": parity,
        "cpu_sw": cpu_sw,
        "seed_roofline": seed_rf,
        "phase_ms": {k: statistics.median(s[k] for s in stats)
                     for k in ("seed_ms", "pairs_ms", "sw_ms", "select_ms", "traceback_ms",
                               "format_ms", "total_ms")},
        "seed_overflow_strands": stats[-1]["seed_overflow_strands"],
        "roofline": {"bound": "dpx", "kernel": rf_kernel,
                     "achieved": achieved, "peak": peak,
                     "unit": "Gcells/s", "frac": achieved / peak if peak and achieved else None,
                     "kernel_ms": rf_ms,
                     "traffic": rf_traffic,
                     "traffic_unit": "bytes per pass (launches of up to 262,144 pairs), "
                                     "ncu DRAM bytes per cell computed x cells computed",
                     "algorithmic_bytes": rf_algo,
                     "peak_source": "measured on this GPU: 2 cells per __vimax3_s16x2_relu "
                                    "lane instruction (%s)" % rf_note,
                     # the same issue-rate peak per ALU-pipe instruction: how busy the
                     # pipe that bounds the kernel is kept
                     "alu_pipe_frac": (achieved / peak * TRACE_ALU_PER_2_CELLS
                                       if tr_ms > 0 and peak and achieved else None)},
        "lcs_bound": None if last["first_pass_kind"] != 3 else {
            "kernel": "sw_lcs_kernel (bit-parallel LCS bound of every packed pair)",
            "kernel_ms": fp_ms, "pairs": fast_pairs,
            "Gcells_per_s": last["first_pass_cells"] / (fp_ms * 1e-3) / 1e9 if fp_ms > 0 else None,
            "pairs_left_for_the_exact_pass": last["lcs_kept"]},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(sum(s["launches"] for s in stats)),
        "clocks": clk.summary(),
        "configs": configs,
    }
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
