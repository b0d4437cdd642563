"""Benchmark: exact Q(N) row-boundary contraction at N=18 on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 18]

One step = one complete exact contraction of Q(N) (all rows, all first-row
orbit slices) through the library's C ABI. Prints one JSON line. By default
the contraction runs with use_graph: the first warm-up step records its row
steps and captures them as one CUDA graph, and every later step replays the
whole contraction on the device from its seeds (checked row by row against the
recorded run); --no-graph contracts eagerly every step.

value  : boundary entries per second = (boundary entries of the merged
         contraction: the sum over rows of the merged frontier's input states)
         / (device time of the whole contraction, CUDA events on the
         library's stream). When the library slices the frontier into device
         batches it processes more entries than that (lost merges); those
         are reported as boundary_entries_processed_per_step and do not
         inflate `value`.
e2e    : the same entries / wall time of the C-ABI call (host seeding,
         host->device upload of the seed boundary, all row steps, device->host
         read-back of every row's metrics and of the count residues).
roofline: the merge step (scatter + merge kernels, plus the row count),
         algorithmic bytes E*(S_in+S_out) summed over the row steps of one
         contraction over those kernels' CUDA-event time; `traffic` is the DRAM
         bytes ncu measured over all scatter and merge launches of one Q(18)
         contraction with the default tuning.
cpu_baseline: the CPU oracle (threaded restatement of the reference's
         sort-reduce driver) on the first rows of the same workload.

--impl reference times only that CPU restatement (there is no runnable
reference binary: the reference is Rust and no Rust toolchain exists here).
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

# Boundary entries of the merged contraction of Q(N): the sum over rows of the
# merged frontier's input states (the reference's LayerMetric.input_states),
# i.e. the work unit of "boundary entries/s", independent of how a run slices
# the frontier. N <= 16 match the CPU oracle; 17 and 18 were measured by this
# library in single-batch merged runs (tail_row off, one device batch).
MERGED_ENTRIES = {16: 397600651, 17: 2684482260, 18: 16682949222}
# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) over every
# partition scatter and merge launch of one contraction, default tuning.
DRAM_TRAFFIC_PER_STEP = {18: 1873.1e9}
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
        "data": "synthetic (empty N x N board)",
        "config": {"workload": f"Q({args.n}) orbit-sliced row contraction, first {args.cpu_rows} rows",
                   "n": args.n, "rows": args.cpu_rows},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"first {args.cpu_rows} rows of Q({args.n}) ({entries} boundary entries), "
                                   f"threaded C++ restatement of contract_rows_d4_orbit_parallel_sort_reduce"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    ctx = pkg.Context(local if world > 1 else 0)
    opts = {"use_graph": 0 if args.no_graph else 1}
    if args.slice_depth:
        opts["slice_depth"] = args.slice_depth
    if args.grain == "site":
        opts["granularity"] = pkg.GRAIN_SITE
    if args.tail_row is not None:
        opts["tail_row"] = args.tail_row

    def barrier():
        if world > 1:
            import torch.distributed as dist  # noqa: PLC0415

            dist.barrier()

    for _ in range(args.warmup):
        r = ctx.contract_rows(args.n, **opts)
        assert r.count == pkg.known_count(args.n)
    barrier()
    sampler = ClockSampler(local if world > 1 else 0)
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

    entries_run = results[-1].device["entries_in"]
    entries = MERGED_ENTRIES.get(args.n, entries_run) if results[-1].device["batches"] > 1 else entries_run
    dev_s = max(sum(x.device["device_ms"] for x in results) / len(results) / 1e3, 1e-12)
    wall_s = max(t_all / args.steps, 1e-12)
    if world > 1:
        dev_s, wall_s = max_over_ranks([dev_s, wall_s], device="cuda")
    if rank != 0:
        return
    value = entries * world / dev_s
    e2e = entries * world / wall_s

    peak, peak_kind = measured_peaks()
    d = results[-1].device
    achieved = d["merge_kernel_bytes"] / max(d["device_ms"] / 1e3, 1e-12) / 1e9
    roofline = {
        "bound": "hbm",
        "kernel": ("merge step: partition_scatter_list_kernel + partition_merge_list_kernel" if d["merge"] == 2
                   else "merge step: row_expand_insert_kernel + compact_kernel (global table)"),
        "achieved": achieved,
        "peak": peak,
        "peak_kind": peak_kind,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": (DRAM_TRAFFIC_PER_STEP.get(args.n) if d["merge"] == 2 and args.grain == "row" else None),
        "traffic_scope": "DRAM bytes per step (one contraction), ncu, all scatter + merge launches",
        "algorithmic_bytes_per_step": d["merge_kernel_bytes"],
        "launches_per_step": d["merge_kernel_launches"],
        "scatter_ms_per_step": d["scatter_kernel_ms"],
        "merge_ms_per_step": d["merge_kernel_ms"],
        "step_ms_per_step": d["device_ms"],
    }
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
        "dtype": f"u{d['key_bits']} keys + {d['residues']}x u32 residues",
        "data": "synthetic (empty N x N board; the workload has no external input)",
        "config": {
            "workload": f"Q({args.n}) exact, all first-row orbit slices",
            "n": args.n,
            "grain": args.grain,
            "slice_depth": d["slice_depth"],
            "batches": d["batches"],
            "residues": d["residues"],
            "key_bits": d["key_bits"],
            "merge": {1: "hash", 2: "partition"}.get(d["merge"], d["merge"]),
            "l2": "inputs larger than L2 (boundary buffers of GBs per row)",
            "parallelism": "replicas" if world > 1 else "single",
            "cuda_graph": not args.no_graph,
        },
        "count": str(results[-1].count),
        "wall_s_per_step": wall_s,
        "device_s_per_step": dev_s,
        "boundary_entries_per_step": entries,
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
        ce, cw, _ = cpu_sample(args.n, args.cpu_rows, threads)
        line["cpu_baseline"] = {
            "value": ce / cw, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {args.cpu_rows} rows of Q({args.n}) ({ce} boundary entries), threaded C++ "
                      f"restatement of contract_rows_d4_orbit_parallel_sort_reduce",
        }
    print(json.dumps(line), flush=True)
    ctx.close()


def run_serve(args):
    """Seeded Poisson stream of counting requests through the continuous-batching
    server. Prints one JSON line: p50/p99 latency and requests/s."""
    import random  # noqa: PLC0415

    world, rank, _ = dist_env()
    if rank != 0:
        return
    pkg = importlib.import_module(PACKAGE)
    if not pkg.LIBRARY_PATH.exists():
        pkg.build()
    rng = random.Random(args.serve_seed)
    reqs = []
    t = 0.0
    for tag in range(args.serve_requests):
        t += rng.expovariate(args.serve_rate)
        n = rng.randint(args.serve_nmin, args.serve_nmax)
        k = rng.randint(0, 3)
        reqs.append((t, tag, n, pkg.random_prefix(rng, n, k)))
    got = {}
    sv = pkg.Server(0, use_cache=int(not args.serve_no_cache))
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
    computed = sorted(c["latency_s"] for c in got.values() if c["path"] != "cache")
    # Exactness (after the timed stream): k = 0 against the known counts; every
    # distinct request with N <= serve_check_nmax against the CPU oracle; a
    # seeded sample of larger boards against the oracle; a sample recomputed
    # alone through a fresh context; the sum rule over all 1-row prefixes.
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
            elif n <= args.serve_check_nmax:
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
        for tag, key in srng.sample(deep, min(args.serve_sample_per_n, len(deep))):
            if key not in want:
                want[key] = oracle_count(*key)
            checked += 1
            sampled += 1
            wrong += int(got[tag]["count"] != want[key] or got[tag]["status"] != 0)
    alone_checked = alone_wrong = 0
    ctx = pkg.Context(0)
    for _, tag, n, prefix in srng.sample(reqs, min(64, len(reqs))):
        if tag in got and n <= 17:
            alone_checked += 1
            alone_wrong += int(ctx.count(n, prefix) != got[tag]["count"])
    n_rule = min(args.serve_nmax, 16)
    rule_sum = sum(ctx.count(n_rule, [c]) for c in range(n_rule))
    ctx.close()
    sum_rule_ok = rule_sum == pkg.known_count(n_rule)
    paths = {}
    for c in got.values():
        paths[c["path"]] = paths.get(c["path"], 0) + 1
    line = {
        "metric": "serve p50/p99 latency (mixed-N prefix counting stream)",
        "value": len(got) / wall,
        "unit": "requests/s",
        "n_gpus": 1,
        "higher_is_better": True,
        "p50_latency_s": q(lat, 0.50),
        "p99_latency_s": q(lat, 0.99),
        "computed_p50_latency_s": q(computed, 0.50),
        "computed_p99_latency_s": q(computed, 0.99),
        "completed": len(got),
        "submitted": len(reqs),
        "wall_s": wall,
        "checked": checked,
        "wrong": wrong,
        "checked_large_sample": sampled,
        "alone_vs_mixed": {"checked": alone_checked, "wrong": alone_wrong},
        "sum_rule": {"n": n_rule, "ok": sum_rule_ok},
        "paths": paths,
        "server": stats,
        "clocks": clocks,
        "config": {"workload": "Poisson stream, N ~ U{%d..%d}, k ~ U{0..3} random legal prefixes"
                   % (args.serve_nmin, args.serve_nmax), "requests": args.serve_requests,
                   "rate_per_s": args.serve_rate, "seed": args.serve_seed, "cache": not args.serve_no_cache},
        "data": "synthetic (seeded request stream)",
    }
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
    ap.add_argument("--tail-row", type=int, default=None,
                    help="first row run by the slice-tail kernel (default: library auto; >= n disables it)")
    ap.add_argument("--cpu-rows", type=int, default=9)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true",
                    help="contract eagerly every step (default: the first warm-up step captures the row steps "
                         "as a CUDA graph and later steps replay it)")
    ap.add_argument("--serve", action="store_true", help="run the serving stream instead of the Q(N) step")
    ap.add_argument("--serve-requests", type=int, default=10000)
    ap.add_argument("--serve-rate", type=float, default=200.0, help="mean arrivals per second")
    ap.add_argument("--serve-seed", type=int, default=20261203)
    ap.add_argument("--serve-nmin", type=int, default=10)
    ap.add_argument("--serve-nmax", type=int, default=19)
    ap.add_argument("--serve-no-cache", action="store_true")
    ap.add_argument("--serve-check-nmax", type=int, default=15)
    ap.add_argument("--serve-sample-per-n", type=int, default=2, help="oracle-checked requests per N above the check limit")
    ap.add_argument("--serve-timeout", type=float, default=900.0)
    args = ap.parse_args()
    if args.serve:
        run_serve(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
