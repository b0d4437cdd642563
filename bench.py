"""Benchmark: exact Q(N) row-boundary contraction at N=18 on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 18]

One step = one complete exact contraction of Q(N) (all rows, all first-row
orbit slices) through the library's C ABI. Prints one JSON line. By default
the contraction runs with use_graph: the first warm-up step records its row
steps and captures them as one CUDA graph, and every later step replays the
whole contraction on the device from its seeds (checked row by row against the
recorded run); --no-graph contracts eagerly every step.

value  : boundary entries per second = (boundary entries of the merged
         contraction: the sum over device rows of the merged frontier's input
         states, the reference's LayerMetric.input_states) / (device time of
         the whole contraction, CUDA events on the library's stream). The
         merged figure is measured in the same run: one untimed contraction
         on a separate context with the whole frontier in one device batch.
         When the timed steps slice the frontier into several device batches
         they process more entries (lost merges); those are reported as
         boundary_entries_processed_per_step and do not inflate `value`.
e2e    : the same entries / wall time of the C-ABI call (host seeding,
         host->device upload of the seed boundary, all row steps, device->host
         read-back of every row's metrics and of the count residues).
roofline: the merge step (scatter + merge kernels), algorithmic bytes
         E*(S_in+S_out) summed over the row steps of one contraction over
         those kernels' CUDA-event time. `traffic` is DRAM bytes per step
         scaled from a small ncu capture of peak-row launches (see
         TRAFFIC_PER_ALGORITHMIC_BYTE); null where none applies.
cpu_baseline: the CPU oracle (threaded restatement of the reference's
         sort-reduce driver) on the first rows of the same workload, median of
         three samples.
same_workload: the full Q(16) contraction on both the GPU (this library) and
         the CPU oracle (all host threads, median of three), so that the two
         rates compare identical work.
serve  : a short seeded Poisson stream through the continuous-batching server
         (--serve runs the full 10,000-request stream on its own).

--impl reference times only that CPU restatement (there is no runnable
reference binary: the reference is Rust and no Rust toolchain exists here),
with the same `config` as this arm and each step a bounded sample of it.
Inputs are synthetic by construction: the workload is the empty N x N board.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

PACKAGE = "quantum-harness-peps-naive_gb300"

# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic
# byte of the merge step, from a capture of the scatter and merge launches of
# rows 11-13 of Q(17) (the peak rows; profiles/dram_q17_peak_rows.md): 171.29 GB
# moved for 56.97 GB of algorithmic bytes. The bench scales the contraction's
# algorithmic bytes by it (an upper estimate: the peak rows re-read the most).
# Keyed by the scatter kind the figure was captured with (1, the window scatter).
TRAFFIC_PER_ALGORITHMIC_BYTE: dict = {1: 171.290302464 / 56.96632816}
METRIC = "Q(N) wall time & boundary entries/s at N=18 (bit-exact)"
UNIT = "boundary entries/s"


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def cpu_sample(n: int, rows: int, threads: int):
    """Oracle (threaded sort-reduce restatement) on the first `rows` rows."""
    import oracle_py  # noqa: PLC0415

    oracle_py.build()
    t0 = time.perf_counter()
    r = oracle_py.contract(n, backend=oracle_py.PARALLEL_SORT_REDUCE, threads=threads, rows=rows)
    wall = time.perf_counter() - t0
    entries = sum(l["input_states"] for l in r["layers"])
    return entries, wall, r


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of per-rank timings over the process group (the
    slowest replica sets the step time)."""
    import torch  # noqa: PLC0415
    import torch.distributed as dist  # noqa: PLC0415

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def workload_config(args) -> dict:
    """The workload both arms report: what is computed, not how this run did it."""
    world, _, _ = dist_env()
    return {
        "workload": f"Q({args.n}) exact, all first-row orbit slices",
        "n": args.n,
        "grain": args.grain,
        "l2": "inputs larger than L2 (boundary buffers of GBs per row)",
        "parallelism": "replicas" if world > 1 else "single",
    }


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(args.n, args.cpu_rows, threads)
    vals, walls, entries = [], [], 0
    for _ in range(args.steps):
        e, w, _ = cpu_sample(args.n, args.cpu_rows, threads)
        vals.append(e / w)
        walls.append(w)
        entries = e
    v = statistics.median(vals)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": statistics.median(walls) * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64 keys + u128 checked coefficients",
        "data": "synthetic (empty N x N board; the workload has no external input)",
        "config": workload_config(args),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"first {args.cpu_rows} rows of Q({args.n}) ({entries} boundary entries) per step, "
                                   f"threaded C++ restatement of contract_rows_d4_orbit_parallel_sort_reduce "
                                   f"(src/lib.rs:5469-5626); median of {args.steps} steps"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def merged_entries(pkg, n: int, device: int, opts: dict):
    """Boundary entries of the merged contraction of Q(n): one untimed
    contraction with the whole frontier in one device batch (slice_depth 1:
    only the first row on the host) on a context of its own, closed
    afterwards. None when that batch does not fit the device."""
    c = pkg.Context(device)
    try:
        r = c.contract_rows(n, slice_depth=1, use_graph=0,
                            **{k: v for k, v in opts.items() if k not in ("use_graph", "slice_depth")})
        if r.count != pkg.known_count(n) or r.device["batches"] != 1:
            return None
        return r.device["entries_in"]
    except pkg.ContractionError:
        return None
    finally:
        c.close()


def same_workload_pair(pkg, ctx, n: int, threads: int, steps: int = 5, cpu_repeats: int = 3) -> dict:
    """Full Q(n) on the GPU (CUDA-graph replay, median wall of `steps`) and on
    the CPU oracle (all host threads, median of `cpu_repeats`)."""
    import oracle_py  # noqa: PLC0415

    ctx.contract_rows(n, use_graph=1)  # records and captures
    walls, devs, r = [], [], None
    for _ in range(steps):
        t0 = time.perf_counter()
        r = ctx.contract_rows(n, use_graph=1)
        walls.append(time.perf_counter() - t0)
        devs.append(r.device["device_ms"] / 1e3)
        assert r.count == pkg.known_count(n)
    entries = r.device["entries_in"] if r.device["batches"] == 1 else None
    oracle_py.build()
    cw = []
    for _ in range(cpu_repeats):
        t0 = time.perf_counter()
        o = oracle_py.contract(n, backend=oracle_py.PARALLEL_SORT_REDUCE, threads=threads)
        cw.append(time.perf_counter() - t0)
        assert o["count"] == pkg.known_count(n)
    cpu_entries = sum(l["input_states"] for l in o["layers"] if l["row"] >= 1)
    gw, gd, cm = statistics.median(walls), statistics.median(devs), statistics.median(cw)
    return {
        "workload": f"Q({n}) exact, all first-row orbit slices, full contraction on both sides",
        "count": str(r.count),
        "gpu_wall_s": gw,
        "gpu_device_s": gd,
        "cpu_wall_s": cm,
        "cpu_wall_s_all": cw,
        "cpu_threads": threads,
        "cpu_kind": "threaded C++ restatement of contract_rows_d4_orbit_parallel_sort_reduce (src/lib.rs:5469-5626)",
        "boundary_entries": entries,
        "cpu_boundary_entries": cpu_entries,
        "gpu_entries_per_s": (entries / gw) if entries else None,
        "cpu_entries_per_s": cpu_entries / cm,
        "wall_speedup": cm / gw,
    }


def run_ours(args):
    world, rank, local = dist_env()
    pkg = importlib.import_module(PACKAGE)
    if not pkg.LIBRARY_PATH.exists():
        pkg.build()
    if world > 1:
        import torch  # noqa: PLC0415
        import torch.distributed as dist  # noqa: PLC0415

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if world > 1 else 0
    opts = {"use_graph": 0 if args.no_graph else 1}
    if args.slice_depth:
        opts["slice_depth"] = args.slice_depth
    if args.grain == "site":
        opts["granularity"] = pkg.GRAIN_SITE
    if args.tail_row is not None:
        opts["tail_row"] = args.tail_row
    if args.key_bits:
        opts["key_bits"] = args.key_bits
    if args.merge:
        opts["merge"] = {"hash": pkg.MERGE_HASH, "partition": pkg.MERGE_PARTITION}[args.merge]
    merged = (merged_entries(pkg, args.n, device, opts)
              if args.grain == "row" and not args.no_merged_run else None)
    ctx = pkg.Context(device)
    tuning_note = None
    if args.tuning_cache and Path(args.tuning_cache).exists():
        tuning_note = ctx.load_tuning(args.n, Path(args.tuning_cache))
    if args.set_tuning:
        kv = dict(item.split("=", 1) for item in args.set_tuning.split(","))
        ctx.set_tuning(**{k: (float(v) if "." in v else int(v)) for k, v in kv.items()})

    def barrier():
        if world > 1:
            import torch.distributed as dist  # noqa: PLC0415

            dist.barrier()

    for _ in range(args.warmup):
        r = ctx.contract_rows(args.n, **opts)
        assert r.count == pkg.known_count(args.n)
    barrier()
    sampler = ClockSampler(device)
    sampler.start()
    results, walls = [], []
    t_all0 = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = ctx.contract_rows(args.n, **opts)
        walls.append(time.perf_counter() - t0)
        if r.count != pkg.known_count(args.n):
            raise SystemExit(f"count mismatch: {r.count} != {pkg.known_count(args.n)}")
        results.append(r)
    t_all = time.perf_counter() - t_all0
    barrier()
    clocks = sampler.stop()

    d = results[-1].device
    entries_run = d["entries_in"]
    if d["batches"] == 1:
        entries, entries_kind = entries_run, "merged (one device batch)"
    elif merged is not None:
        entries, entries_kind = merged, "merged (measured in this run, one untimed single-batch contraction)"
    else:
        entries, entries_kind = entries_run, "processed (the merged figure could not be measured)"
    dev_s = max(sum(x.device["device_ms"] for x in results) / len(results) / 1e3, 1e-12)
    wall_s = max(t_all / args.steps, 1e-12)
    if world > 1:
        dev_s, wall_s = max_over_ranks([dev_s, wall_s], device="cuda")
    if rank != 0:
        return
    value = entries * world / dev_s
    e2e = entries * world / wall_s

    peak, peak_kind = measured_peaks()
    achieved = d["merge_kernel_bytes"] / max(d["device_ms"] / 1e3, 1e-12) / 1e9
    tuning = ctx.tuning
    kind = tuning.get("scatter_kind")
    # The capture behind the factor is of the u64 row path's scatter and merge.
    tpb = (TRAFFIC_PER_ALGORITHMIC_BYTE.get(kind)
           if d["merge"] == 2 and args.grain == "row" and d["key_bits"] == 64 else None)
    roofline = {
        "bound": "hbm",
        "kernel": ("merge step: partition scatter + partition merge kernels" if d["merge"] == 2
                   else "merge step: row_expand_insert_kernel + compact_kernel (global table)"),
        "achieved": achieved,
        "peak": peak,
        "peak_kind": peak_kind,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": (tpb * d["merge_kernel_bytes"]) if tpb else None,
        "traffic_scope": ("DRAM bytes per step: the step's algorithmic bytes x 3.007, the DRAM bytes per algorithmic "
                          "byte that ncu measured on the scatter and merge launches of Q(17) rows 11-13 (an upper "
                          "estimate)" if tpb else "no capture for this configuration"),
        "algorithmic_bytes_per_step": d["merge_kernel_bytes"],
        "launches_per_step": d["merge_kernel_launches"],
        "scatter_ms_per_step": d["scatter_kernel_ms"],
        "merge_ms_per_step": d["merge_kernel_ms"],
        "step_ms_per_step": d["device_ms"],
        # Successor candidates per step, and per second of scatter-kernel time
        # (summed over concurrent lanes, so a per-kernel rate).
        "candidates_per_step": d["candidates"],
        "scatter_candidates_per_s": d["candidates"] / max(d["scatter_kernel_ms"] / 1e3, 1e-12),
    }
    if d["exact_weights"]:
        dtype = f"u{d['key_bits']} keys + exact u64 weights (2x u32 words), host-side CRT bookkeeping"
    else:
        dtype = f"u{d['key_bits']} keys + {d['residues']}x u32 residues"
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wall_s * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": dtype,
        "data": "synthetic (empty N x N board; the workload has no external input)",
        "config": workload_config(args),
        "run": {
            "slice_depth": d["slice_depth"],
            "batches": d["batches"],
            "residues": d["residues"],
            "exact_weights": bool(d["exact_weights"]),
            "key_bits": d["key_bits"],
            "merge": {1: "hash", 2: "partition"}.get(d["merge"], d["merge"]),
            "cuda_graph": not args.no_graph,
            "tuning": tuning,
            "tuning_cache": tuning_note,
        },
        "count": str(results[-1].count),
        **({"layers": [[l.row, l.input_states, l.completed_row_terms, l.output_states] for l in results[-1].layers]}
           if args.layers else {}),
        "wall_s_per_step": wall_s,
        "device_s_per_step": dev_s,
        "boundary_entries_per_step": entries,
        "boundary_entries_kind": entries_kind,
        "boundary_entries_processed_per_step": entries_run,
        "peak_states": results[-1].peak_states,
        "peak_device_bytes": d["peak_device_bytes"],
        "gpu_launches": sum(x.device["gpu_launches"] for x in results),
        "clocks": clocks,
        "roofline": roofline,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": d["h2d_bytes"],
                "d2h_bytes_per_step": d["d2h_bytes"]},
    }
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        samples = [cpu_sample(args.n, args.cpu_rows, threads)[:2] for _ in range(3)]
        rates = [e / w for e, w in samples]
        line["cpu_baseline"] = {
            "value": statistics.median(rates), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {args.cpu_rows} rows of Q({args.n}) ({samples[0][0]} boundary entries), threaded C++ "
                      f"restatement of contract_rows_d4_orbit_parallel_sort_reduce (src/lib.rs:5469-5626); "
                      f"median of 3 samples",
            "samples": rates,
        }
        if args.same_workload_n:
            line["same_workload"] = same_workload_pair(pkg, ctx, args.same_workload_n, threads)
    if world == 1 and d["merge"] == 2 and d["key_bits"] == 64 and not args.no_pattern_probe:
        # The scatter's access pattern alone on this device (random 16-byte
        # appends into hash partitions, one cursor atomic each), measured
        # after the timed region: the time the step's candidates need at that
        # rate bounds the merge step from below, whatever the DRAM bandwidth.
        cand = 512 << 20
        fill = float(tuning.get("partition_fill", 0.75))
        parts = int(cand / (fill * 2048)) + 1
        try:
            rate = cand / (ctx.probe_append(pkg.PROBE_APPEND, cand, parts, repeats=3) * 1e-3)
        except pkg.ContractionError as e:  # e.g. too little free device memory for the probe's regions
            line["scatter_pattern"] = {"unavailable": e.message}
        else:
            bound_ms = d["candidates"] / rate * 1e3
            line["scatter_pattern"] = {
                "pattern": "random 16-byte appends into hash partitions of 2048 slots, one cursor atomic each",
                "probe_records": cand, "probe_partitions": parts, "probe_records_per_s": rate,
                "candidates_per_step": d["candidates"], "pattern_bound_ms_per_step": bound_ms,
                "step_ms_per_step": d["device_ms"], "frac": bound_ms / max(d["device_ms"], 1e-12),
            }
    ctx.close()
    if world == 1 and args.dfs_check:
        # The DFS bitboard oracle (src/dfs_bitmask.rs:67-340, restated in C++)
        # on all host threads, run in the same job as an independent check.
        import oracle_py  # noqa: PLC0415

        oracle_py.build()
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        dfs = oracle_py.dfs_count(args.n, threads=threads)
        line["dfs_check"] = {"count": str(dfs), "equal": dfs == results[-1].count, "wall_s": time.perf_counter() - t0,
                             "threads": threads}
    if world == 1 and args.serve_requests_inline:
        line["serve"] = serve_stream(pkg, args, requests=args.serve_requests_inline, check_nmax=13,
                                     sample_per_n=0, alone_samples=16, compact=True)
    print(json.dumps(line), flush=True)


def serve_stream(pkg, args, requests: int, check_nmax: int, sample_per_n: int, alone_samples: int,
                 compact: bool = False) -> dict:
    """Seeded Poisson stream of counting requests through the
    continuous-batching server; latency percentiles, throughput and exactness
    checks (after the timed stream)."""
    import random  # noqa: PLC0415

    rng = random.Random(args.serve_seed)
    reqs = []
    t = 0.0
    for tag in range(requests):
        t += rng.expovariate(args.serve_rate)
        n = rng.randint(args.serve_nmin, args.serve_nmax)
        k = rng.randint(0, 3)
        reqs.append((t, tag, n, pkg.random_prefix(rng, n, k)))
    got = {}
    cfg = {"use_cache": int(not args.serve_no_cache)}
    if args.serve_large_workers:
        cfg["large_workers"] = args.serve_large_workers
    sv = pkg.Server(0, **cfg)
    sampler = ClockSampler(0)
    sampler.start()
    t0 = time.perf_counter()
    for at, tag, n, prefix in reqs:
        while True:
            now = time.perf_counter() - t0
            if now >= at:
                break
            for c in sv.poll(wait_ms=max(0, min(5, int((at - now) * 1e3)))):
                got[c["tag"]] = c
        sv.submit(n, prefix, tag)
    deadline = time.perf_counter() + args.serve_timeout
    while len(got) < len(reqs) and time.perf_counter() < deadline:
        for c in sv.poll(wait_ms=50):
            got[c["tag"]] = c
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    stats = sv.stats()
    sv.close()
    lat = sorted(c["latency_s"] for c in got.values())
    q = lambda xs, f: xs[min(len(xs) - 1, int(f * len(xs)))] if xs else None  # noqa: E731
    computed = sorted(c["latency_s"] for c in got.values() if c["path"] not in ("cache", "coalesced"))
    # Exactness: k = 0 against the known counts; every distinct request with
    # N <= check_nmax against the CPU oracle; a seeded sample of larger boards
    # against the oracle; a sample recomputed alone through a fresh context;
    # the sum rule over all 1-row prefixes.
    import oracle_py  # noqa: PLC0415

    oracle_py.build()
    threads = os.cpu_count() or 1

    def oracle_count(n, prefix):
        return oracle_py.contract(n, backend=oracle_py.PARALLEL_SORT_REDUCE, symmetry=False, threads=threads,
                                  prefix=prefix)["count"]

    want = {}
    checked = wrong = 0
    big = []
    for _, tag, n, prefix in reqs:
        c = got.get(tag)
        if c is None:
            continue
        key = (n, tuple(prefix))
        if key not in want:
            if not prefix:
                want[key] = pkg.known_count(n)
            elif n <= check_nmax:
                want[key] = oracle_count(n, prefix)
            else:
                big.append((tag, key))
                continue
        checked += 1
        wrong += int(c["count"] != want[key] or c["status"] != 0)
    srng = random.Random(args.serve_seed + 1)
    by_n = {}
    for tag, key in big:
        by_n.setdefault(key[0], []).append((tag, key))
    sampled = 0
    for n in sorted(by_n):
        pool = sorted(by_n[n], key=lambda tk: -len(tk[1][1]))  # deepest prefixes first: smallest frontiers
        deep = [tk for tk in pool if len(tk[1][1]) == len(pool[0][1][1])]
        for tag, key in srng.sample(deep, min(sample_per_n, len(deep))):
            if key not in want:
                want[key] = oracle_count(*key)
            checked += 1
            sampled += 1
            wrong += int(got[tag]["count"] != want[key] or got[tag]["status"] != 0)
    alone_checked = alone_wrong = 0
    ctx = pkg.Context(0)
    for _, tag, n, prefix in srng.sample(reqs, min(alone_samples, len(reqs))):
        if tag in got and n <= 17:
            alone_checked += 1
            alone_wrong += int(ctx.count(n, prefix) != got[tag]["count"])
    n_rule = min(args.serve_nmax, 16)
    rule_sum = sum(ctx.count(n_rule, [c]) for c in range(n_rule))
    ctx.close()
    paths = {}
    for c in got.values():
        paths[c["path"]] = paths.get(c["path"], 0) + 1
    out = {
        "metric": "serve p50/p99 latency (mixed-N prefix counting stream)",
        "value": len(got) / wall,
        "unit": "requests/s",
        "computed_p50_latency_s": q(computed, 0.50),
        "computed_p99_latency_s": q(computed, 0.99),
        "computed_requests": len(computed),
        "p50_latency_s": q(lat, 0.50),
        "p99_latency_s": q(lat, 0.99),
        "completed": len(got),
        "submitted": len(reqs),
        "wall_s": wall,
        "checked": checked,
        "wrong": wrong,
        "checked_large_sample": sampled,
        "alone_vs_mixed": {"checked": alone_checked, "wrong": alone_wrong},
        "sum_rule": {"n": n_rule, "ok": rule_sum == pkg.known_count(n_rule)},
        "paths": paths,
        "server": stats,
        "config": {"workload": "Poisson stream, N ~ U{%d..%d}, k ~ U{0..3} random legal prefixes"
                   % (args.serve_nmin, args.serve_nmax), "requests": requests,
                   "rate_per_s": args.serve_rate, "seed": args.serve_seed, "cache": not args.serve_no_cache,
                   "large_workers": args.serve_large_workers or "default"},
    }
    if not compact:
        out["clocks"] = clocks
        out["n_gpus"] = 1
        out["higher_is_better"] = True
        out["data"] = "synthetic (seeded request stream)"
    return out


def run_serve(args):
    """The full serving stream; one JSON line."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    pkg = importlib.import_module(PACKAGE)
    if not pkg.LIBRARY_PATH.exists():
        pkg.build()
    line = serve_stream(pkg, args, requests=args.serve_requests, check_nmax=args.serve_check_nmax,
                        sample_per_n=args.serve_sample_per_n, alone_samples=64)
    print(json.dumps(line), flush=True)


def run_explicit(args):
    """The explicit-C site frontier (contract_explicit_c_frontier,
    src/lib.rs:961-967) at one N and order, through the partitioned merge
    (default) and through the global table; one JSON line, wall time of the
    default path as the value."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    pkg = importlib.import_module(PACKAGE)
    if not pkg.LIBRARY_PATH.exists():
        pkg.build()
    order = {"row": pkg.ORDER_ROW_MAJOR, "diamond": pkg.ORDER_TOP_LEFT_DIAMOND}[args.explicit_order]
    fields = ("count", "complete", "peak_states", "peak_open_bonds", "tensor_entries_examined",
              "tensor_entries_accepted", "contracted_sites")
    arms = {}
    for name, merge in (("partition", pkg.MERGE_PARTITION), ("hash", pkg.MERGE_HASH)):
        ctx = pkg.Context(0)
        ctx.set_tuning(merge_auto=merge)
        for _ in range(args.warmup):
            ctx.explicit_frontier(args.explicit, order, args.explicit_limit)
        walls, dev = [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            r = ctx.explicit_frontier(args.explicit, order, args.explicit_limit)
            walls.append(time.perf_counter() - t0)
            dev.append(r["device_ms"])
        ctx.close()
        arms[name] = {"wall_ms": statistics.median(walls) * 1e3, "device_ms": statistics.median(dev),
                      "gpu_launches": r["gpu_launches"], **{k: r[k] for k in fields}}
    same = all(arms["partition"][k] == arms["hash"][k] for k in fields)
    line = {"metric": "explicit-C site frontier wall time", "value": arms["partition"]["wall_ms"], "unit": "ms",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False,
            "dtype": "u128 keys + u32 residues", "data": "none (the count of the N x N board)",
            "config": {"workload": "explicit-C site frontier, N=%d, %s order" % (args.explicit, args.explicit_order),
                       "support_limit": args.explicit_limit},
            "count": str(arms["partition"]["count"]), "partition_equals_hash": same, "arms": arms}
    print(json.dumps(line, default=str), flush=True)
    if not same:
        sys.exit(1)


def run_probe(args):
    """The partition scatter's memory pattern alone (qpeps_probe_append):
    random 16-byte appends with one cursor atomic each, the stores without the
    atomics, the atomics without the stores, and coalesced stores, at the
    scatter's partition sizing; one JSON line with each mode's best rate."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    pkg = importlib.import_module(PACKAGE)
    if not pkg.LIBRARY_PATH.exists():
        pkg.build()
    ctx = pkg.Context(0)
    cases = []
    for cand in args.probe_candidates:
        parts = max(1, int(cand / (args.probe_fill * 2048)) + 1)
        row = {"candidates": cand, "parts": parts, "fill": args.probe_fill}
        for name, mode in (("append", pkg.PROBE_APPEND), ("store_only", pkg.PROBE_STORE),
                           ("atomic_only", pkg.PROBE_ATOMIC), ("stream", pkg.PROBE_STREAM),
                           ("append_plain", pkg.PROBE_APPEND_PLAIN)):
            ms = ctx.probe_append(mode, cand, parts, repeats=args.steps)
            row[name] = {"ms": ms, "records_per_s": cand / (ms * 1e-3), "gb_per_s": cand * 16 / (ms * 1e-3) / 1e9}
        cases.append(row)
    ctx.close()
    line = {"metric": "partition scatter pattern rate (16-byte records into hash partitions)", "unit": "records/s",
            "value": cases[0]["append"]["records_per_s"], "n_gpus": 1, "steps": args.steps, "warmup": 1,
            "higher_is_better": True, "data": "synthetic (pseudo-random keys)",
            "config": {"workload": "random appends into partitions of 2048 16-byte slots", "fill": args.probe_fill},
            "cases": cases}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=18)
    ap.add_argument("--grain", choices=["row", "site"], default="row")
    ap.add_argument("--slice-depth", type=int, default=0)
    ap.add_argument("--key-bits", type=int, choices=[0, 64, 128], default=0,
                    help="boundary key width (0: the library's choice, u64 up to N=21)")
    ap.add_argument("--merge", choices=["", "hash", "partition"], default="",
                    help="merge strategy (default: the library's choice)")
    ap.add_argument("--tail-row", type=int, default=None,
                    help="first row run by the slice-tail kernel (default: library auto; >= n disables it)")
    ap.add_argument("--cpu-rows", type=int, default=9)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--layers", action="store_true",
                    help="add each row's [row, input states, successor terms, output states] of the last step")
    ap.add_argument("--no-merged-run", action="store_true",
                    help="skip the untimed single-batch contraction that measures the merged entries")
    ap.add_argument("--dfs-check", action="store_true",
                    help="after timing, count Q(n) with the CPU DFS bitboard oracle on all host threads")
    ap.add_argument("--same-workload-n", type=int, default=16,
                    help="full Q(n) on both the GPU and the CPU oracle beside the headline (0: skip)")
    ap.add_argument("--tuning-cache", default=str(ROOT / PACKAGE / "tuning_gb300.json"),
                    help="autotuner cache (JSON) whose entry for this device and N is applied before timing")
    ap.add_argument("--set-tuning", default="",
                    help="tuning fields applied before timing, e.g. scatter_kind=3,unit_target=1000")
    ap.add_argument("--no-graph", action="store_true",
                    help="contract eagerly every step (default: the first warm-up step captures the row steps "
                         "as a CUDA graph and later steps replay it)")
    ap.add_argument("--probe", action="store_true",
                    help="time the partition scatter's memory pattern alone instead of the Q(N) step")
    ap.add_argument("--probe-candidates", type=int, nargs="+", default=[64 << 20, 512 << 20])
    ap.add_argument("--probe-fill", type=float, default=0.75)
    ap.add_argument("--no-pattern-probe", action="store_true",
                    help="leave the scatter-pattern probe out of the Q(N) line")
    ap.add_argument("--explicit", type=int, default=0,
                    help="time the explicit-C site frontier at this N instead of the Q(N) step")
    ap.add_argument("--explicit-order", choices=["row", "diamond"], default="diamond")
    ap.add_argument("--explicit-limit", type=int, default=5_000_000, help="support limit of the explicit-C frontier")
    ap.add_argument("--serve", action="store_true", help="run the serving stream instead of the Q(N) step")
    ap.add_argument("--serve-requests", type=int, default=10000)
    ap.add_argument("--serve-requests-inline", type=int, default=1000,
                    help="requests of the short stream reported in the default line (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="mean arrivals per second")
    ap.add_argument("--serve-seed", type=int, default=20261203)
    ap.add_argument("--serve-nmin", type=int, default=10)
    ap.add_argument("--serve-nmax", type=int, default=19)
    ap.add_argument("--serve-no-cache", action="store_true")
    ap.add_argument("--serve-large-workers", type=int, default=0,
                    help="concurrent large-request contexts of the server (0: library default)")
    ap.add_argument("--serve-check-nmax", type=int, default=15)
    ap.add_argument("--serve-sample-per-n", type=int, default=2, help="oracle-checked requests per N above the check limit")
    ap.add_argument("--serve-timeout", type=float, default=900.0)
    args = ap.parse_args()
    if args.serve:
        run_serve(args)
    elif args.probe:
        run_probe(args)
    elif args.explicit:
        run_explicit(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
