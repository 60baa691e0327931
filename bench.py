#!/usr/bin/env python3
"""Throughput of PaKman's k-mer counting -> histogram cutoff -> macro-node path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload bacterial|plain|longk] [--scale S]

One step = one pass of the whole path (count, cutoff, macro-nodes) over one read
set.  The default workload is the 4.6 Mbp genome / 80x / 100 bp / k=32 read set
(seeded synthetic reads, ~254M k-mer windows).  `value` is k-mer windows per
second with the FASTA bytes already resident in HBM; `e2e` is the same metric
through the C ABI with the FASTA in pinned host memory and the macro-node table
copied back every step.  Under torchrun each rank runs an independent replica
(the path has no cross-device exchange on one GPU per job); value = all ranks'
windows / max rank time.
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

METRIC = "k-mers/sec count+macro-node on 1 GB300 (% HBM roofline); served p50/p99 latency"
UNIT = "k-mers/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["bacterial", "plain", "longk"], default="bacterial")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--e2e-workers", type=int, default=4,
                    help="jobs in flight in the end-to-end (serving API) measurement")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-windows", type=int, default=0,
                    help="windows in the CPU baseline's sample (0: the whole read set)")
    ap.add_argument("--bucket-bits", type=int, default=0, help="partition digits (0 = automatic)")
    ap.add_argument("--compact-threshold", type=int, default=100000,
                    help="node threshold of the compaction measurement (the reference's -n default)")
    ap.add_argument("--no-compaction", action="store_true")
    ap.add_argument("--compact-cpu-scale", type=float, default=0.1,
                    help="genome scale of the compaction CPU baseline's sample")
    ap.add_argument("--batch", action="store_true",
                    help="batching benchmark: many read sets in one CUDA-graph launch")
    ap.add_argument("--batch-sets", type=int, default=256)
    ap.add_argument("--batch-branches", type=int, default=6)
    ap.add_argument("--batch-check-every", type=int, default=8,
                    help="every n-th set of the batch is checked against the oracle")
    ap.add_argument("--serve", action="store_true",
                    help="serving benchmark: Poisson stream of jobs through pk_submit, p50/p99 latency")
    ap.add_argument("--serve-jobs", type=int, default=5000)
    ap.add_argument("--serve-rate", type=float, default=200.0, help="mean arrivals per second")
    ap.add_argument("--serve-pool", type=int, default=32, help="distinct generated read sets")
    ap.add_argument("--serve-workers", type=int, default=12)
    ap.add_argument("--serve-budget-gb", type=float, default=160.0)
    ap.add_argument("--serve-small-sms", type=int, default=16,
                    help="SMs set aside for small requests in the SM-partition run")
    ap.add_argument("--serve-reserved-small", type=int, default=4,
                    help="workers that take only small requests (-1: the library's default)")
    ap.add_argument("--serve-modes", default="host,resident,partition",
                    help="which streams to run: host (tables to pinned host memory), resident, partition")
    ap.add_argument("--ingest", action="store_true",
                    help="file ingest benchmark: FASTA file -> macro-node table on the host, read "
                         "into memory then counted, against streamed by pk_count_file")
    return ap.parse_args()


def workload(name: str, scale: float):
    from pakman_plus_gb300 import synth
    return {"bacterial": synth.config2, "plain": synth.config1, "longk": synth.config3}[name](scale)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id):
        self.lines = []
        self.proc = None
        self.bus_id = bus_id

    def start(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.bus_id:
            cmd += ["-i", self.bus_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def stage_bytes(stage: str, F: int, N: int, U: int, V: int, M: int, W: int, t: int, B: int,
                G: int) -> int:
    """Algorithmic bytes one launch of a stage must move (read + write)."""
    return {
        "line_scan": F,
        # the counting pass also writes each 16-byte unit packed (10 bytes), which the
        # coarse scatter reads instead of the FASTA
        "bucket_count": F + 5 * F // 8 + 4 * G * B,
        "bucket_offsets": 3 * 4 * G * B,
        "scatter_coarse": 5 * F // 8 + N * W,
        "scatter_fine": 2 * N * W,
        "bucket_table": N * W + U * (W + 4),
        "cutoff": 8 * t,
        "kept_filter": U * (W + 4) + V * (W + 4),
        "macro_nodes": 2 * V * (W + 4) + M * (W + 32),
    }.get(stage, 0)


def pipeline_bytes(F, N, U, V, M, W):
    """Whole-path model: F + 2NW + 2U(W+4) + 4U + 4V(W+4) + M(W+32)."""
    return F + 2 * N * W + 2 * U * (W + 4) + 4 * U + 4 * V * (W + 4) + M * (W + 32)


def _cpu_sample(rs, sample_windows: int):
    """The first reads of the workload holding about `sample_windows` windows (0: all)."""
    if sample_windows <= 0:
        return rs.fasta, rs.n_reads
    per_read = max(1, rs.read_len - rs.k + 1)
    reads = min(rs.n_reads, max(1, sample_windows // per_read))
    if reads >= rs.n_reads:
        return rs.fasta, rs.n_reads
    lines = rs.fasta.split(b"\n")
    return b"\n".join(lines[: 2 * reads]) + b"\n", reads


def cpu_baseline(rs, sample_windows: int):
    """The oracle's multi-threaded restatement of the reference's owner-partitioned
    counting (all host cores) plus cutoff and macro-nodes, on the same read set.
    Returns the baseline line and the oracle's result when the sample is the whole read
    set (else None)."""
    from oracle import pk_oracle as po
    sample, reads = _cpu_sample(rs, sample_windows)
    threads = os.cpu_count() or 1
    po.lib()
    t0 = time.perf_counter()
    pipe = po.run(sample, rs.k, rs.t, rs.drop_n, threads=threads)
    dt = time.perf_counter() - t0
    n = pipe.table.n_windows
    line = {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{reads} reads ({n} k-mer windows) of the same read set, count + cutoff + "
                      f"macro-nodes, {dt:.2f} s on {threads} threads"}
    return line, (pipe if reads == rs.n_reads else None)


def _digest(*arrays) -> str:
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(a.tobytes())
    return h.hexdigest()[:16]


def device_result(job, rs):
    """The device's whole result for the bench's read set: table, histogram, cutoff and
    macro-node table (the macro-nodes are built again, so the job is left at stage 3)."""
    import pakman_plus_gb300 as pk
    keys, counts = job.table()
    cut, hist, kept = job.cutoff(rs.t)
    job.build_macro_nodes(0)
    mn = job.macro_nodes()
    return {"keys": pk.to_key128(keys), "counts": counts, "cutoff": cut, "hist": hist,
            "mn_keys": pk.to_key128(mn.keys), "mn_suf": mn.suffix_counts, "mn_pre": mn.prefix_counts}


def parity(dev, pipe, scale: float):
    """Bit-exact comparison of the device result with the oracle's on the same reads."""
    import numpy as np
    table = bool(dev["keys"].size == pipe.table.keys.size and
                 np.array_equal(dev["keys"], pipe.table.keys) and
                 np.array_equal(dev["counts"], pipe.table.counts))
    mn = pipe.mn is not None and bool(
        dev["mn_keys"].size == pipe.mn.keys.size and np.array_equal(dev["mn_keys"], pipe.mn.keys) and
        np.array_equal(dev["mn_suf"], pipe.mn.suf) and np.array_equal(dev["mn_pre"], pipe.mn.pre))
    return {"table": table, "cutoff": bool(dev["cutoff"] == pipe.cutoff),
            "hist": bool(np.array_equal(dev["hist"], pipe.hist)), "mn": bool(mn), "scale": scale,
            "rows": int(dev["keys"].size), "nodes": int(dev["mn_keys"].size),
            "table_sha256_16": _digest(dev["keys"], dev["counts"]),
            "oracle_table_sha256_16": _digest(pipe.table.keys, pipe.table.counts),
            "mn_sha256_16": _digest(dev["mn_keys"], dev["mn_suf"], dev["mn_pre"]),
            "oracle_mn_sha256_16": (_digest(pipe.mn.keys, pipe.mn.suf, pipe.mn.pre)
                                    if pipe.mn is not None else None),
            "against": "the oracle's threaded restatement (equal to the serial oracle, which is "
                       "pinned to the reference) on the same reads, whole read set"}


def max_over_ranks(x: float, dist, device: str) -> float:
    """The slowest rank's time (every rank gets it); `dist` is None for one process."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(windows_per_rank: int, world: int, ms: float) -> float:
    """Whole-job k-mers/s: every replica counts its own read set of the same size, so
    the job processes world x windows in the slowest rank's time."""
    return windows_per_rank * world / (ms / 1000.0)


def measure_compaction(job, rs, args, M, reps=3):
    """Iterative compaction (pk_compact) of this workload's macro-node table down to
    --compact-threshold nodes: device time of the whole call (CUDA events around it on
    the job's stream, host round trips between rounds included), median of `reps`."""
    import ctypes

    from pakman_plus_gb300 import capi
    L = capi.lib()
    info = capi.PkCompactionInfo()

    def once():
        st = L.pk_compact(job.handle, args.compact_threshold, rs.coverage, ctypes.byref(info))
        if st != 0:
            raise RuntimeError("pk_compact: " + L.pk_last_error().decode())
        return job.stage_times()["compaction"]

    once()
    l0 = L.pk_kernel_launches()
    ms = statistics.median(once() for _ in range(reps))
    compact_launches = (L.pk_kernel_launches() - l0) / reps
    winfo = capi.PkWalkInfo()

    def walk_once():
        st = L.pk_walk(job.handle, ctypes.byref(winfo))
        if st != 0:
            raise RuntimeError("pk_walk: " + L.pk_last_error().decode())
        return job.stage_times()["walk"]

    walk_once()
    l0 = L.pk_kernel_launches()
    wms = statistics.median(walk_once() for _ in range(reps))
    walk_launches = (L.pk_kernel_launches() - l0) / reps
    return {"workload": f"{rs.name} macro-node table -> at most {args.compact_threshold} nodes",
            "nodes_in": int(M), "nodes_out": int(info.n_nodes), "rounds": int(info.rounds),
            "partial_contigs": int(info.n_contigs), "ms": ms, "nodes_per_s": M / (ms / 1000.0),
            "launches": compact_launches,
            "launches_per_round": compact_launches / max(1, int(info.rounds)),
            "walk": {"ms": wms, "begin_kmers": int(winfo.n_begins), "contigs": int(winfo.n_contigs),
                     "contig_bases": int(winfo.contig_bases), "launches": walk_launches},
            "nodes_per_s_with_walk": M / ((ms + wms) / 1000.0)}


def compaction_cpu_baseline(name, scale, threshold):
    """The oracle's C restatement of compaction + walk (oracle/pk_compact.c, one
    thread; the reference's own compaction is serial) on a scaled sample of the same
    workload, its node threshold scaled alike: macro-nodes per second."""
    import pakman_plus_gb300 as pk
    from oracle import pk_compact as pc
    rs = workload(name, scale)
    p = pk.default_params(k=rs.k, num_buckets=rs.t, coverage=rs.coverage, drop_n=int(rs.drop_n))
    ctx = pk.Context(0)
    with pk.Job(ctx) as job:
        job.count(rs.fasta, p)
        job.cutoff(rs.t)
        job.build_macro_nodes(0)
        mn = job.macro_nodes(rs.coverage)
    ctx.close()
    t0 = time.perf_counter()
    r = pc.compact_walk_c(mn.keys, mn.suffix_counts, mn.prefix_counts, rs.k, rs.coverage, threshold)
    sec = time.perf_counter() - t0
    return {"value": len(mn.keys) / sec, "unit": "macro-nodes/s", "cores": 1, "kind": "port",
            "sample": f"{rs.name} at scale {scale}: {len(mn.keys)} macro-nodes -> {r.n_nodes} in {r.rounds} "
                      f"rounds, then the walk ({r.walk_contigs} contigs), {sec:.2f} s; compare with the "
                      f"device's compaction + walk time"}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return 0
    rs = workload(args.workload, args.scale)
    from oracle import pk_oracle as po
    sample, reads = _cpu_sample(rs, args.cpu_sample_windows)
    exe = po.build_reference(rs.k) if os.path.isdir(po.REFERENCE_TREE) else None
    if exe is None:
        exe_path = os.path.join(po.REF_OUT, f"pakman_ref_k{rs.k}")
        exe = exe_path if os.path.exists(exe_path) and os.access(exe_path, os.X_OK) else None
    kind = "reference" if exe else "port"
    threads = os.cpu_count() or 1
    po.lib()
    times, n_windows = [], 0
    for step in range(args.warmup + args.steps):
        if kind == "reference":
            r = po.run_reference(sample, rs.k, rs.read_len, rs.coverage, rs.t, threads=threads,
                                 want_mn=False)
            dt = r.seconds.get("count_s", 0.0) + r.seconds.get("mn_s", 0.0)
            n_windows = int(r.table_counts.sum())
        else:
            t0 = time.perf_counter()
            pipe = po.run(sample, rs.k, rs.t, rs.drop_n, threads=threads)
            dt = time.perf_counter() - t0
            n_windows = pipe.table.n_windows
        if step >= args.warmup:
            times.append(dt)
    ms = 1000.0 * sum(times) / len(times)
    value = n_windows / (ms / 1000.0)
    cores = threads
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64" if rs.k <= 32 else "u128",
            "data": "synthetic",
            "config": {"workload": rs.name, "reads": rs.n_reads, "read_len": rs.read_len, "k": rs.k,
                       "t": rs.t, "sample_reads": reads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"first {reads} reads ({n_windows} k-mer windows) per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _mn_digest(keys, suf, pre) -> str:
    import hashlib
    h = hashlib.sha256()
    for x in (keys, suf, pre):
        h.update(memoryview(x).cast("B"))
    return h.hexdigest()[:16]


def run_serve(args, rank, world):
    """Serving workload: jobs (genome log-uniform 10 kb-20 Mbp, 100 bp reads at 30-80x,
    k in {31, 32, 63}) arrive as a Poisson stream and go through pk_submit/pk_wait
    with HBM-budget admission and size-aware scheduling; the same stream is then served
    one job at a time (the plain one-job-per-launch path), and both are run again with
    every job submitted at once (capacity at saturation).  A pool of generated read sets
    stands in for the stream's inputs (job i uses pool entry i mod P with that entry's
    k).  Every pool entry's result is checked against the oracle (table and macro-nodes),
    every served job's summary against its entry's, and one served table per entry
    byte for byte."""
    if rank != 0:
        return 0
    import threading

    import numpy as np
    import torch

    import pakman_plus_gb300 as pk
    from oracle import pk_oracle as po
    from pakman_plus_gb300 import build as pkbuild
    from pakman_plus_gb300 import synth

    pkbuild.build()
    torch.cuda.set_device(0)
    t_gen = time.perf_counter()
    pool, pinned, params, pool_bytes = [], [], [], 0
    for i in range(args.serve_pool):  # generated and pinned one at a time
        rs = synth.config5_job(i)
        pool.append(rs)
        buf = torch.empty(len(rs.fasta), dtype=torch.uint8, pin_memory=True)
        buf.numpy()[:] = np.frombuffer(rs.fasta, np.uint8)
        pinned.append(buf)
        pool_bytes += len(rs.fasta)
        params.append(pk.default_params(k=rs.k, num_buckets=21, coverage=rs.coverage, read_length=100))
        rs.fasta = b""  # the pinned copy is the input from here on
    t_gen = time.perf_counter() - t_gen
    budget = int(args.serve_budget_gb * 1e9)
    ctx = pk.Context(0, hbm_budget=budget)
    # each pool entry alone, once: reference summaries, macro-node digests and warm-up
    # (a job whose k-mers all fall below the cutoff ends with PK_ERR_EMPTY, as the
    # reference aborts; that outcome must then be the same in the stream)
    alone, alone_digest, oracle_ok = [], [], []
    t_ora = 0.0
    threads = os.cpu_count() or 1
    device_ms = []  # kernel time of each entry alone (CUDA events around its stages)
    with pk.Job(ctx) as job:
        for e, rs in enumerate(pool):
            t0 = time.perf_counter()
            status = 0
            mn = None
            try:
                job.run(pinned[e].numpy(), params[e])
                mn = job.macro_nodes()
            except pk.EmptyAfterCutoff as ex:
                status = ex.status
            alone.append((job.summary(), time.perf_counter() - t0, status))
            keys, counts = job.table()
            alone_digest.append(_mn_digest(mn.keys, mn.suffix_counts, mn.prefix_counts) if mn else None)
            t1 = time.perf_counter()
            ora = po.run(pinned[e].numpy().tobytes(), rs.k, 21, threads=threads)
            t_ora += time.perf_counter() - t1
            k128 = pk.to_key128(keys)
            ok = k128.size == ora.table.keys.size and np.array_equal(k128, ora.table.keys) and \
                np.array_equal(counts, ora.table.counts) and alone[-1][0].cutoff == ora.cutoff
            if ora.mn is None:
                ok = ok and status != 0
            else:
                ok = ok and mn is not None and np.array_equal(pk.to_key128(mn.keys), ora.mn.keys) and \
                    np.array_equal(mn.suffix_counts, ora.mn.suf) and np.array_equal(mn.prefix_counts, ora.mn.pre)
            oracle_ok.append(bool(ok))
            del ora, keys, counts, mn
            # a second, timed run: the first launch of each kernel loads its module
            job.enable_timing(True)
            try:
                job.run(pinned[e].numpy(), params[e])
            except pk.EmptyAfterCutoff:
                pass
            stages = job.stage_times()
            device_ms.append(sum(v for k, v in stages.items() if k != "h2d"))
            job.enable_timing(False)
            job.reset()
    # each entry's solo latency through the server (nothing else in flight), best of two,
    # with the table copied to pinned host memory and with it kept on the device
    solo, solo_res = [], []
    srv = pk.Server(ctx, workers=args.serve_workers)
    for e in range(len(pool)):
        for keep, out in ((False, solo), (True, solo_res)):
            best = None
            for _ in range(2):
                tk = srv.submit(pinned[e].numpy(), params[e], keep_on_device=keep)
                try:
                    srv.wait(tk)
                except pk.PakmanError:
                    pass
                lat = srv.poll(tk).latency_ms
                srv.release(tk)
                best = lat if best is None else min(best, lat)
            out.append(best)
    srv.close()
    rng = np.random.Generator(np.random.PCG64(5_000_001))
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, args.serve_jobs))
    entries = [i % len(pool) for i in range(args.serve_jobs)]

    def serve(workers, arrival, resident=False, small_sms=0):
        """The stream through a server of `workers` workers; `resident`: every table stays
        on the device (keep_on_device) until the consumer releases it, instead of the
        macro-node table crossing to pinned host memory; `small_sms`: SMs set aside for
        small requests (an SM partition)."""
        rsv = args.serve_reserved_small if args.serve_reserved_small >= 0 and workers > 1 else None
        srv = pk.Server(ctx, workers=workers, small_sms=small_sms, reserved_small=rsv)
        partition = srv.partition()
        tickets = [None] * args.serve_jobs
        by_ticket = {}

        def producer():
            t0 = time.perf_counter()
            for i, e in enumerate(entries):
                dt = t0 + arrival[i] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                t = srv.submit(pinned[e].numpy(), params[e], keep_on_device=resident)
                tickets[i] = t
                by_ticket[t] = i

        th = threading.Thread(target=producer, daemon=True)
        th.start()
        lat, ratio, first_submit, last_end, windows, mismatches = [], [], None, 0, 0, 0
        small_ratio, large_ratio = [], []
        # results are taken in completion order and released at once, so the server's
        # pinned result blocks are recycled whatever order it ran the jobs in
        for _ in entries:
            info = srv.next_done()
            while info.ticket not in by_ticket:  # the producer has not recorded it yet
                time.sleep(0.0002)
            i = by_ticket[info.ticket]
            e = entries[i]
            ref, _, ref_status = alone[e]
            s = info.summary
            if info.status != ref_status or (s.n_windows, s.n_unique, s.n_kept, s.cutoff) != (
                    ref.n_windows, ref.n_unique, ref.n_kept, ref.cutoff) or (
                    ref_status == 0 and s.n_nodes != ref.n_nodes):
                mismatches += 1
            srv.release(info.ticket)
            lat.append(info.latency_ms)
            ratio.append(info.latency_ms / (solo_res[e] if resident else solo[e]))
            (small_ratio if pinned[e].numel() * (2 if params[e].k > 32 else 1) <= (32 << 20)
             else large_ratio).append(ratio[-1])
            first_submit = info.submit_ns if first_submit is None else min(first_submit, info.submit_ns)
            last_end = max(last_end, info.end_ns)
            windows += s.n_windows
        th.join()
        st = srv.stats()
        srv.close()
        lat, ratio = np.array(lat), np.array(ratio)
        span = (last_end - first_submit) / 1e9
        return {"workers": workers, "results": "resident on the device" if resident else "pinned host memory",
                "sm_partition": {"small_requests": partition[0], "others": partition[1]} if small_sms else None,
                "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                "max_ms": float(lat.max()), "p50_latency_over_solo": float(np.percentile(ratio, 50)),
                "p99_latency_over_solo": float(np.percentile(ratio, 99)),
                "jobs_within_2x_solo": float((ratio <= 2.0).mean()),
                "small_jobs": {"jobs": len(small_ratio),
                               "p50_latency_over_solo": float(np.percentile(small_ratio, 50)) if small_ratio else None,
                               "p99_latency_over_solo": float(np.percentile(small_ratio, 99)) if small_ratio else None},
                "large_jobs": {"jobs": len(large_ratio),
                               "p50_latency_over_solo": float(np.percentile(large_ratio, 50)) if large_ratio else None,
                               "p99_latency_over_solo": float(np.percentile(large_ratio, 99)) if large_ratio else None},
                "kmers_per_s": windows / span, "span_s": span,
                "peak_admitted_gb": st["peak_admitted_bytes"] / 1e9, "requeued": st["requeued"],
                "worker_s_by_phase": {ph: round(st[ph + "_ns"] / 1e9, 3)
                                      for ph in ("count", "cutoff", "mn", "copyout", "release", "pin")},
                "results_differing_from_alone": mismatches}

    def tables_in_the_mix():
        """Every pool entry served among the others (all submitted at once, twice over)
        gives the macro-node table of the entry run alone, byte for byte."""
        srv = pk.Server(ctx, workers=args.serve_workers)
        order = list(range(len(pool))) * 2
        tickets = [srv.submit(pinned[e].numpy(), params[e]) for e in order]
        differing = 0
        for tk, e in zip(tickets, order):
            try:
                srv.wait(tk)
                mn = srv.result(tk)
                d = _mn_digest(mn.keys, mn.suffix_counts, mn.prefix_counts)
            except pk.EmptyAfterCutoff:
                d = None
            differing += d != alone_digest[e]
            srv.release(tk)
        srv.close()
        return {"jobs": len(order), "macro_node_tables_differing": differing}

    def link_gbps():
        """Host-to-device copy rate of the largest pool entry right now (best of three):
        the host link is shared with the machine's other tenants, and every request's
        input crosses it."""
        e = max(range(len(pool)), key=lambda i: pinned[i].numel())
        dst = torch.empty(pinned[e].numel(), dtype=torch.uint8, device="cuda")
        best = float("inf")
        for _ in range(3):
            torch.cuda.synchronize()
            t = time.perf_counter()
            dst.copy_(pinned[e], non_blocking=True)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t)
        del dst
        return pinned[e].numel() / best / 1e9

    modes = set(args.serve_modes.split(","))
    skipped = {"skipped": "not in --serve-modes"}
    mix_check = tables_in_the_mix()
    link_before = link_gbps()
    at_once = np.zeros(args.serve_jobs)
    served = plain = served_sat = plain_sat = skipped
    if "host" in modes:
        served = serve(args.serve_workers, arrivals)
        plain = serve(1, arrivals)
        served_sat = serve(args.serve_workers, at_once)
        plain_sat = serve(1, at_once)
    link_after = link_gbps()
    # tables kept on the device: no macro-node table crosses the host link
    served_res = served_res_sat = plain_res_sat = skipped
    if "resident" in modes:
        served_res = serve(args.serve_workers, arrivals, resident=True)
        served_res_sat = serve(args.serve_workers, at_once, resident=True)
        plain_res_sat = serve(1, at_once, resident=True)
    # small requests on SMs of their own (green contexts), tables resident
    part = part_sat = skipped
    if "partition" in modes:
        try:
            part = serve(args.serve_workers, arrivals, resident=True, small_sms=args.serve_small_sms)
            part_sat = serve(args.serve_workers, at_once, resident=True, small_sms=args.serve_small_sms)
        except pk.PakmanError as ex:
            part = part_sat = {"unavailable": str(ex)}

    def ratio_of(a, b):
        return a["kmers_per_s"] / b["kmers_per_s"] if "kmers_per_s" in a and "kmers_per_s" in b else None
    total_windows = sum(alone[e][0].n_windows for e in entries)
    offered = total_windows / arrivals[-1]
    # what the GPU could serve if the stream's kernels ran back to back with nothing
    # between them: every job's windows over the sum of its kernel time alone
    device_bound = total_windows / (sum(device_ms[e] for e in entries) / 1e3)
    small_windows = sum(alone[e][0].n_windows for e in entries
                        if pinned[e].numel() * (2 if params[e].k > 32 else 1) <= (32 << 20))
    headline = served if "p99_ms" in served else served_res
    line = {"metric": "served p50/p99 latency of count + macro-node jobs", "impl": "serve",
            "value": headline.get("p99_ms"), "unit": "ms (p99)", "higher_is_better": False,
            "n_gpus": 1, "data": "synthetic",
            "config": {"workload": "serving: Poisson arrivals, genome log-uniform 10 kb-20 Mbp, 100 bp reads "
                                   "at 30-80x, 0.5% errors, k in {31,32,63}",
                       "jobs": args.serve_jobs, "rate_per_s": args.serve_rate, "pool_read_sets": len(pool),
                       "pool_fasta_gb": pool_bytes / 1e9, "pool_gen_s": t_gen,
                       "hbm_budget_gb": args.serve_budget_gb,
                       "offered_kmers_per_s": offered,
                       "alone_ms_by_entry": [round(a[1] * 1000, 2) for a in alone],
                       "solo_served_ms_by_entry": [round(x, 2) for x in solo],
                       "solo_resident_ms_by_entry": [round(x, 2) for x in solo_res],
                       "device_ms_by_entry": [round(x, 3) for x in device_ms],
                       "link_h2d_gbps_before_after_streams": [round(link_before, 1), round(link_after, 1)],
                       "device_bound_kmers_per_s": device_bound,
                       "small_jobs_kmer_share": small_windows / total_windows,
                       "entries_empty_after_cutoff": sum(1 for a in alone if a[2] != 0)},
            "oracle": {"entries_equal": sum(oracle_ok), "entries": len(oracle_ok), "seconds": t_ora,
                       "against": "table, cutoff and macro-nodes of every pool entry against the oracle's "
                                  f"threaded restatement ({threads} threads)"},
            "tables_in_the_mix": mix_check,
            "served": served, "plain_one_job_at_a_time": plain,
            "saturation": {"served": served_sat, "plain_one_job_at_a_time": plain_sat,
                           "capacity_ratio": ratio_of(served_sat, plain_sat),
                           "served_over_device_bound": served_sat["kmers_per_s"] / device_bound
                           if "kmers_per_s" in served_sat else None},
            "resident_sm_partition": {"served": part, "saturation": part_sat},
            "resident": {"served": served_res,
                         "saturation": {"served": served_res_sat, "plain_one_job_at_a_time": plain_res_sat,
                                        "capacity_ratio": ratio_of(served_res_sat, plain_res_sat),
                                        "served_over_device_bound": served_res_sat["kmers_per_s"] / device_bound
                                        if "kmers_per_s" in served_res_sat else None}}}
    print(json.dumps(line), flush=True)
    ctx.close()
    bad = sum(not x for x in oracle_ok) + mix_check["macro_node_tables_differing"] + sum(
        r.get("results_differing_from_alone", 0) for r in (served, plain, served_sat, plain_sat, served_res,
                                                           served_res_sat, plain_res_sat, part, part_sat))
    if bad:
        print("bench: served results differ from the oracle or from the jobs run alone", file=sys.stderr)
        return 3
    return 0


def run_batch(args, rank, world):
    """Batching workload: independent read sets (genome log-uniform 20 kb-5 Mbp, reads
    of 100-150 bp at 20-80x, 0.5% errors, k=32) in one CUDA-graph launch per step,
    against the same sets run one job at a time with their input already in HBM."""
    if rank != 0:
        return 0
    import numpy as np
    import torch

    import pakman_plus_gb300 as pk
    from pakman_plus_gb300 import build as pkbuild
    from pakman_plus_gb300 import synth

    pkbuild.build()
    torch.cuda.set_device(0)
    t_gen = time.perf_counter()
    sets, pinned, total_bytes = [], [], 0
    for i in range(args.batch_sets):
        rs = synth.config4_set(i, args.scale)
        buf = torch.empty(len(rs.fasta), dtype=torch.uint8, pin_memory=True)
        buf.numpy()[:] = np.frombuffer(rs.fasta, np.uint8)
        pinned.append(buf)
        total_bytes += len(rs.fasta)
        sets.append((buf.numpy(), pk.default_params(k=32, num_buckets=21, coverage=rs.coverage,
                                                    read_length=rs.read_len)))
    t_gen = time.perf_counter() - t_gen
    ctx = pk.Context(0)
    # device value: the sets copied before the graph, so the launch runs with its inputs
    # in HBM
    batch = pk.Batch(ctx, branches=args.batch_branches, input_in_graph=False)
    res = batch.run(sets)  # autotune + capture + first launch
    st0 = batch.stats()
    windows = sum(r.summary.n_windows for r in res)
    graph_ms = []
    for _ in range(max(1, args.warmup)):
        batch.run(sets)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = batch.run(sets)
        graph_ms.append(batch.stats()["last_graph_ms"])
    wall_before = (time.perf_counter() - t0) / args.steps
    # end to end: the graph copies each pinned set itself, overlapping other branches
    batch.set_input_in_graph(True)
    for _ in range(max(1, args.warmup)):
        batch.run(sets)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = batch.run(sets)
    wall = (time.perf_counter() - t0) / args.steps
    keys, suf, pre = batch.table()
    st = batch.stats()
    # the plain path: one job per set, inputs already on the device
    dev = [torch.from_numpy(f).cuda() for f, _ in sets]
    plain_ms = []
    with pk.Job(ctx) as job:
        job.enable_timing(False)
        for rep in range(2):
            torch.cuda.synchronize()
            t = time.perf_counter()
            for d, (_, p) in zip(dev, sets):
                try:
                    job.run_device(d.data_ptr(), d.numel(), p)
                except pk.EmptyAfterCutoff:
                    pass
            torch.cuda.synchronize()
            plain_ms.append(1000 * (time.perf_counter() - t))
    med = sorted(graph_ms)[len(graph_ms) // 2]
    tuned_shapes = {}
    for f, _ in sets:
        cls = "%d KiB" % ((1 << (len(f).bit_length() - 1)) >> 10)
        try:
            tuned_shapes[cls] = "digits %d, chunk x%d, table CTAs/SM %d" % batch.tuned_shape(len(f), 32)
        except pk.PakmanError:
            tuned_shapes[cls] = "not tuned"
    # every 8th set (32 of 256, spread over the size range) against the oracle: summary,
    # cutoff and the set's rows of the batch's macro-node table
    from oracle import pk_oracle as po
    threads = os.cpu_count() or 1
    checked, equal = 0, 0
    t_ora = time.perf_counter()
    for i in range(0, len(sets), max(1, args.batch_check_every)):
        f, p = sets[i]
        ora = po.run(f.tobytes(), 32, 21, threads=threads)
        r = res[i]
        ok = r.summary.n_unique == ora.table.keys.size and r.summary.n_windows == ora.table.n_windows
        if ora.mn is None:
            ok = ok and r.status != 0
        else:
            mn = batch.macro_nodes(r, (keys, suf, pre), p.coverage)
            ok = ok and r.status == 0 and r.summary.cutoff == ora.cutoff and \
                np.array_equal(pk.to_key128(mn.keys), ora.mn.keys) and \
                np.array_equal(mn.suffix_counts, ora.mn.suf) and np.array_equal(mn.prefix_counts, ora.mn.pre)
        checked += 1
        equal += bool(ok)
    t_ora = time.perf_counter() - t_ora
    line = {"metric": "batched count + macro-node k-mers/s (one CUDA-graph launch per batch)", "impl": "batch",
            "value": windows / (med / 1000.0), "unit": "k-mers/s", "higher_is_better": True, "n_gpus": 1,
            "data": "synthetic", "dtype": "u64",
            "config": {"workload": f"{args.batch_sets} read sets, genome log-uniform 20 kb-5 Mbp, 100-150 bp "
                                   f"reads at 20-80x, 0.5% errors, k=32", "scale": args.scale,
                       "fasta_gb": total_bytes / 1e9, "kmer_windows": windows, "branches": args.batch_branches,
                       "gen_s": t_gen},
            "graph_ms": med, "graph_launches_per_step": 1,
            "kernels_per_launch": st["kernels_per_launch"], "captures": st["graph_captures"],
            "reruns": st["reruns"], "tuned_classes": st["tuned_classes"], "tune_ms": st["tune_ms"],
            "first_run_ms": st0["last_graph_ms"],
            "tuned_shapes": tuned_shapes,
            "e2e": {"value": windows / wall, "unit": "k-mers/s", "ms_per_step": 1000 * wall,
                    "h2d_bytes_per_step": total_bytes,
                    "note": "pk_batch_run from pinned host buffers: the graph copies each set on its branch "
                            "ahead of its kernels, per-set results (table copy separate)",
                    "copied_before_the_graph": {"value": windows / wall_before, "ms_per_step": 1000 * wall_before}},
            "plain_one_job_at_a_time": {"kmers_per_s": windows / (min(plain_ms) / 1000.0),
                                        "ms": min(plain_ms)},
            "statuses": {str(s): sum(1 for r in res if r.status == s) for s in set(r.status for r in res)},
            "total_nodes": st["total_nodes"],
            "oracle": {"sets_checked": checked, "sets_equal": equal, "seconds": t_ora,
                       "against": "summary, cutoff and macro-node rows of every "
                                  f"{args.batch_check_every}th set against the oracle ({threads} threads)"}}
    print(json.dumps(line), flush=True)
    batch.close()
    ctx.close()
    if equal != checked:
        print("bench: batched results differ from the oracle", file=sys.stderr)
        return 3
    return 0


def run_ingest(args, rank, world):
    """FASTA file -> macro-node table in host memory, two ways, on one GPU: (a) the file
    read into pinned host memory, then pk_run (copy, count, cutoff, macro-nodes); (b)
    pk_count_file, whose reader threads stream the file to the device while earlier
    pieces are copied and line-scanned, then cutoff and macro-nodes.  Both copy the
    macro-node table back.  The file is read once before timing, so both read it from
    the page cache; the timings are host wall-clock per file."""
    if rank != 0:
        return 0
    import numpy as np
    import torch

    import pakman_plus_gb300 as pk
    from pakman_plus_gb300 import build as pkbuild

    pkbuild.build()
    rs = workload(args.workload, args.scale)
    F = len(rs.fasta)
    tmpdir = tempfile.mkdtemp(prefix="pk_ingest_")
    path = os.path.join(tmpdir, "reads.fa")
    with open(path, "wb") as f:
        f.write(rs.fasta)
    with open(path, "rb") as f:
        while f.read(1 << 26):
            pass
    params = pk.default_params(k=rs.k, num_buckets=rs.t, coverage=rs.coverage, read_length=rs.read_len,
                               drop_n=int(rs.drop_n), batch_kmers=rs.batch)
    ctx = pk.Context(0)
    pinned = torch.empty(F, dtype=torch.uint8, pin_memory=True).numpy()
    with pk.Job(ctx) as job:  # macro-node count, to size the pinned output buffers
        cap = job.run(rs.fasta, params).n_nodes + 16
    kd = pk.key_dtype(rs.k)
    out = (torch.empty(cap * kd.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(kd),
           torch.empty(cap * 16, dtype=torch.uint8, pin_memory=True).numpy().view(np.uint32).reshape(cap, 4),
           torch.empty(cap * 16, dtype=torch.uint8, pin_memory=True).numpy().view(np.uint32).reshape(cap, 4))

    def read_only():
        with open(path, "rb") as f:
            return f.readinto(memoryview(pinned))

    def via_memory(job):
        n = read_only()
        s = job.run(pinned[:n], params)
        job.macro_nodes(out=out)
        return s

    def via_file(job):
        job.count_file(path, params)
        job.cutoff(rs.t)
        job.build_macro_nodes(0)
        job.macro_nodes(out=out)
        return job.summary()

    def timed(fn, *a):
        t0 = time.perf_counter()
        r = fn(*a)
        return r, (time.perf_counter() - t0) * 1e3

    res = {"read_only": [], "memory": [], "file": []}
    with pk.Job(ctx) as job:
        for step in range(args.warmup + args.steps):
            _, t_read = timed(read_only)
            sm, t_mem = timed(via_memory, job)
            sf, t_file = timed(via_file, job)
            assert (sm.n_windows, sm.n_unique, sm.n_kept, sm.n_nodes) == (sf.n_windows, sf.n_unique, sf.n_kept,
                                                                         sf.n_nodes)
            if step >= args.warmup:
                res["read_only"].append(t_read)
                res["memory"].append(t_mem)
                res["file"].append(t_file)
    med = {k: statistics.median(v) for k, v in res.items()}
    line = {"metric": "file_to_macro_nodes_ms", "impl": "ours", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": False, "data": "synthetic",
            "value": round(med["file"], 3), "unit": "ms",
            "memory_path_ms": round(med["memory"], 3), "file_read_only_ms": round(med["read_only"], 3),
            "file_read_gbs": round(F / med["read_only"] / 1e6, 2),
            "kmers_per_s_file_path": sm.n_windows / (med["file"] * 1e-3),
            "config": {"workload": rs.name, "fasta_bytes": F, "kmer_windows": sm.n_windows,
                       "page_cache": "warm", "host_threads": os.cpu_count()}}
    print(json.dumps(line), flush=True)
    os.remove(path)
    os.rmdir(tmpdir)
    ctx.close()
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    if args.serve:
        return run_serve(args, rank, world)
    if args.batch:
        return run_batch(args, rank, world)
    if args.ingest:
        return run_ingest(args, rank, world)

    import numpy as np
    import torch

    import pakman_plus_gb300 as pk
    from pakman_plus_gb300 import build as pkbuild

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkbuild.build()
    rs = workload(args.workload, args.scale)
    F = len(rs.fasta)
    host = torch.frombuffer(bytearray(rs.fasta), dtype=torch.uint8)
    d_fa = host.to(f"cuda:{local}")
    ctx = pk.Context(local)
    stream = torch.cuda.Stream(device=local)
    job = pk.Job(ctx, stream=stream.cuda_stream)
    params = pk.default_params(k=rs.k, num_buckets=rs.t, coverage=rs.coverage, read_length=rs.read_len,
                               drop_n=int(rs.drop_n), batch_kmers=rs.batch,
                               bucket_bits=args.bucket_bits)
    job.enable_timing(True)
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        s = job.run_device(d_fa.data_ptr(), F, params)
    props = torch.cuda.get_device_properties(local)
    bus = None
    try:
        bus = "%08x:%02x:%02x.0" % (props.pci_domain_id, props.pci_bus_id, props.pci_device_id)
    except AttributeError:
        pass
    sampler = ClockSampler(bus)
    stage_acc = {}
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    launches0 = pk.capi.lib().pk_kernel_launches()
    e0.record(stream)
    for _ in range(args.steps):
        s = job.run_device(d_fa.data_ptr(), F, params)
        for name, ms in job.stage_times().items():
            stage_acc[name] = stage_acc.get(name, 0.0) + ms
    e1.record(stream)
    torch.cuda.synchronize()
    launches = pk.capi.lib().pk_kernel_launches() - launches0
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ms_step = e0.elapsed_time(e1) / args.steps
    ms_step = max_over_ranks(ms_step, dist, f"cuda:{local}")
    value = job_throughput(s.n_windows, world, ms_step)
    dev = device_result(job, rs) if rank == 0 and world == 1 and not args.no_cpu_baseline else None
    compaction = None
    if not args.no_compaction and rank == 0:
        compaction = measure_compaction(job, rs, args, s.n_nodes)

    # end to end through the public API: pinned host FASTA in, macro-node table out,
    # every step; requests go through the serving front end (pk_submit / pk_wait) with
    # `e2e_workers` jobs in flight, so one job's copies overlap another's kernels
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else max(4, min(args.steps, 12))
    depth = max(1, args.e2e_workers)
    pinned = torch.empty(F, dtype=torch.uint8, pin_memory=True)
    pinned.copy_(host)
    pin_np = pinned.numpy()
    W = 8 if rs.k <= 32 else 16
    cap = max(1, 2 * s.n_kept)

    def pinned_out():
        keys = torch.empty(cap * W, dtype=torch.uint8, pin_memory=True).numpy().view(
            np.uint64 if W == 8 else pk.KEY128)
        suf = torch.empty(cap * 16, dtype=torch.uint8, pin_memory=True).numpy().view(np.uint32).reshape(cap, 4)
        pre = torch.empty(cap * 16, dtype=torch.uint8, pin_memory=True).numpy().view(np.uint32).reshape(cap, 4)
        return keys, suf, pre

    outs = [pinned_out() for _ in range(depth)]
    # one job, one request at a time (no overlap), for reference
    job.run(pin_np, params)
    job.macro_nodes(out=outs[0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(2):
        job.run(pin_np, params)
        job.macro_nodes(out=outs[0])
    serial_ms = 1000.0 * (time.perf_counter() - t0) / 2
    job.reset()
    srv = pk.Server(ctx, workers=depth, reserved_small=0)  # every worker takes this size
    for tk in [srv.submit(pin_np, params, out=outs[i]) for i in range(depth)]:  # warm-up
        srv.wait(tk)
        srv.release(tk)
    if dist:
        dist.barrier()
    tickets = []
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        if i >= depth:
            srv.wait(tickets[i - depth])
        tickets.append(srv.submit(pin_np, params, out=outs[i % depth]))
    infos = [srv.wait(tk) for tk in tickets[-depth:]]
    t1 = time.perf_counter()
    lat = sorted((srv.poll(tk).end_ns - srv.poll(tk).start_ns) / 1e6 for tk in tickets)
    se = infos[-1].summary
    srv.close()
    e2e_ms = 1000.0 * (t1 - t0) / e2e_steps
    e2e_ms = max_over_ranks(e2e_ms, dist, f"cuda:{local}")
    e2e = {"value": job_throughput(se.n_windows, world, e2e_ms), "unit": UNIT,
           "h2d_bytes_per_step": F, "d2h_bytes_per_step": int(se.n_nodes * (W + 32) + 48),
           "ms_per_step": e2e_ms, "steps": e2e_steps,
           "mode": f"pk_submit/pk_wait, {depth} jobs in flight, pinned host buffers",
           "job_ms_p50": lat[len(lat) // 2], "serial_ms_per_step": serial_ms}

    if rank == 0:
        peak, peak_kind = peaks()
        U, V, M, N = s.n_unique, s.n_kept, s.n_nodes, s.n_windows
        B = 1 << 15
        G = props.multi_processor_count
        avg = {k: v / args.steps for k, v in stage_acc.items()}
        kern = {k: v for k, v in avg.items() if k != "h2d" and v > 0}
        dom = max(kern, key=kern.get)
        dom_bytes = stage_bytes(dom, F, N, U, V, M, W, rs.t, B, G)
        achieved = dom_bytes / (kern[dom] / 1000.0) / 1e9
        traffic = None
        tp = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tp):
            tj = json.load(open(tp))
            ent = tj.get(rs.name, {}).get(dom)
            if ent:
                traffic = ent.get("dram_bytes_per_launch")
        pb = pipeline_bytes(F, N, U, V, M, W)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64" if rs.k <= 32 else "u128",
            "data": "synthetic",
            "config": {"workload": rs.name, "genome_bp": rs.genome_len, "reads": rs.n_reads,
                       "read_len": rs.read_len, "k": rs.k, "t": rs.t, "coverage": rs.coverage,
                       "fasta_bytes": F, "kmer_windows": N, "distinct_kmers": U, "kept_kmers": V,
                       "macro_nodes": M, "cutoff": s.cutoff, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (FASTA and key buffers > 126 MB)",
                       "pipeline_bytes_model": pb,
                       "pipeline_hbm_frac": pb / (ms_step / 1000.0) / 1e9 / peak,
                       "stage_ms": {k: round(v, 4) for k, v in avg.items()}},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_source": f"{peak_kind} copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"},
            "e2e": e2e,
            "gpu_launches": int(launches),
            "gpu_launches_per_step": launches / args.steps,
            "clocks": clocks,
        }
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"], pipe = cpu_baseline(rs, args.cpu_sample_windows)
            if pipe is not None and dev is not None:
                line["parity"] = parity(dev, pipe, args.scale)
        if compaction is not None:
            if world == 1 and not args.no_cpu_baseline:
                try:
                    compaction["cpu_baseline"] = compaction_cpu_baseline(
                        args.workload, args.compact_cpu_scale,
                        max(1, int(args.compact_threshold * args.compact_cpu_scale)))
                except Exception as e:  # the baseline is reported, never required
                    compaction["cpu_baseline"] = {"unavailable": str(e)[:200]}
            line["compaction"] = compaction
        print(json.dumps(line), flush=True)
    job.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()
    par = line.get("parity") if rank == 0 else None
    if par is not None and not all(par[x] for x in ("table", "cutoff", "hist", "mn")):
        print("bench: the device result differs from the oracle's", file=sys.stderr)
        return 3
    return 0


if __name__ == "__main__":
    sys.exit(main())
