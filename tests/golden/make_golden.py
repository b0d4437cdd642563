"""Regenerate tests/golden/reference_golden.json from the reference tree.

    python tests/golden/make_golden.py /path/to/reference

Reads only the reference's own published values for the row-boundary
contraction path (nothing is computed here):

* known_count Q(0..27)                     src/lib.rs:5752-5784
* orbit-path per-row frontier sizes        benchmarks/e35_frontier_audit_layers.csv
* orbit/dense peak support + work counters benchmarks/e12_d4_orbit_slicing_release.csv
* dense peak support + work counters       benchmarks/current_scaling_peps_release.csv
* N=16 orbit peak support + matched work   benchmarks/e36_joint_u64_release.csv
* dense per-row layers at N=14 (sitewise)  benchmarks/n14_layers.csv
* naive dense HashMap N=14..16 peak        benchmarks/issue34_same_node_algorithm_comparison_scnet.csv
* CRT known answers                        src/lib.rs:3767, 6530-6545; benchmarks/scnet_e50_scaling_n1_n19_release.csv
* explicit-C generic frontier (row-major and top-left diamond site orders):
  count, peak support, peak open bonds, tensor entries examined/accepted,
  contracted sites for N=7..12                benchmarks/e34_corner_frontier_release.csv
"""
from __future__ import annotations

import csv
import json
import re
import sys
from pathlib import Path


def main(ref: Path) -> None:
    lib = (ref / "src/lib.rs").read_text()
    m = re.search(r"const COUNTS: \[u128; 28\] = \[(.*?)\];", lib, re.S)
    known = [int(x.strip().replace("_", "")) for x in m.group(1).split(",") if x.strip()]
    assert len(known) == 28

    m = re.search(r"const CRT_PRIME_CANDIDATES: \[u64; 4\] = \[(.*?)\];", lib, re.S)
    crt_primes = [int(x.strip().replace("_", "")) for x in m.group(1).split(",") if x.strip()]
    m = re.search(r"let value = ([0-9_]+)_u128;", lib)
    crt_kat_value = int(m.group(1).replace("_", ""))

    bench = ref / "benchmarks"
    orbit_layers: dict[str, list[int]] = {}
    with open(bench / "e35_frontier_audit_layers.csv") as f:
        for row in csv.DictReader(f):
            orbit_layers.setdefault(row["N"], []).append(int(row["reachable_states"]))

    def summary(path: Path, key: str) -> dict:
        out: dict = {}
        with open(path) as f:
            for row in csv.DictReader(f):
                out.setdefault(row[key], {})[row["N"]] = {
                    "count": int(row["count"]),
                    "peak_support": int(row["peak_support"]),
                    "row_operator_candidates": int(row["row_operator_candidates"]),
                    "row_operator_matched": int(row["row_operator_matched"]),
                    "threads": int(row["threads"]),
                }
        return out

    e12 = summary(bench / "e12_d4_orbit_slicing_release.csv", "backend")
    dense = summary(bench / "current_scaling_peps_release.csv", "backend")

    e36 = {}
    with open(bench / "e36_joint_u64_release.csv") as f:
        for row in csv.DictReader(f):
            if row["variant"] == "e36_joint_u64":
                e36[row["N"]] = {
                    "count": int(row["count"]),
                    "peak_support": int(row["peak_support"]),
                    "row_operator_matched": int(row["row_operator_matched"]),
                    "max_coefficient_observed": int(row["max_coefficient_observed"]),
                }

    n14 = []
    with open(bench / "n14_layers.csv") as f:
        for row in csv.DictReader(f):
            n14.append({k: int(v) if k != "elapsed_s" else float(v) for k, v in row.items() if k != "peak_rss_bytes"})

    naive = {}
    with open(bench / "issue34_same_node_algorithm_comparison_scnet.csv") as f:
        for row in csv.DictReader(f):
            if row["algorithm_key"] == "naive_peps":
                naive[row["N"]] = {"count": int(row["count"]), "peak_support": int(row["peak_sparse_support"])}

    crt_n19 = None
    with open(bench / "scnet_e50_scaling_n1_n19_release.csv") as f:
        for row in csv.reader(f):
            if row and row[0] == "19":
                primes = [int(x) for x in row[13].split("|")]
                residues = [int(x) for x in row[14].split("|")]
                crt_n19 = {"count": int(row[3]), "primes": primes, "residues": residues}

    explicit = {}
    with open(bench / "e34_corner_frontier_release.csv") as f:
        for row in csv.DictReader(f):
            explicit.setdefault(row["order"], {})[row["N"]] = {
                k: int(row[k])
                for k in ("count", "peak_support", "peak_open_bonds", "tensor_entries_examined",
                          "tensor_entries_accepted", "contracted_sites", "total_sites", "support_limit")
            }
            explicit[row["order"]][row["N"]]["complete"] = row["complete"] == "true"

    golden = {
        "source": "EricNie2003/quantum-harness-peps-naive (reference tree), values copied from files listed in make_golden.py",
        "known_count": [str(v) for v in known],
        "orbit_layers_output_states": orbit_layers,
        "e12_summary": e12,
        "dense_summary": dense,
        "e36_orbit_n16": e36,
        "n14_dense_sitewise_layers": n14,
        "naive_dense_hashmap": naive,
        "explicit_frontier": explicit,
        "crt": {
            "candidate_primes": crt_primes,
            "kat_value_q27": str(crt_kat_value),
            "plan_primes": {"22": 3, "28": 4},
            "n19_scnet": crt_n19,
        },
    }
    out = Path(__file__).resolve().parent / "reference_golden.json"
    out.write_text(json.dumps(golden, indent=1, sort_keys=True) + "\n")
    print(f"wrote {out}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/reference")
    main(Path(sys.argv[1]))
