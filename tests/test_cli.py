"""The qpeps CLI mirrors the reference's binary (src/main.rs:25-174)."""
from __future__ import annotations

import subprocess

import pytest

from conftest import ROOT

CLI = ROOT / "quantum-harness-peps-naive_gb300" / "qpeps"


def _run(*args):
    return subprocess.run([str(CLI), *args], capture_output=True, text=True, timeout=600)


@pytest.fixture(scope="module")
def cli(qp):
    if not CLI.exists():
        qp.build()
    assert CLI.exists()
    return CLI


def test_usage_and_argument_errors(cli):
    r = _run()
    assert r.returncode == 1
    assert "Usage:" in r.stderr and "error: missing or invalid command" in r.stderr
    r = _run("solve", "abc")
    assert r.returncode == 1 and "error: invalid N" in r.stderr
    r = _run("solve")
    assert r.returncode == 1 and "error: missing N" in r.stderr
    r = _run("bench", "9", "--frobnicate")
    assert r.returncode == 1 and "error: unknown option: --frobnicate" in r.stderr
    r = _run("bench", "9", "--repeats", "0")
    assert r.returncode == 1 and "error: --repeats must be positive" in r.stderr
    r = _run("bench", "9", "--min", "10")
    assert r.returncode == 1 and "error: --min must not exceed MAX_N" in r.stderr


@pytest.mark.gpu
def test_solve_line_and_layers_match_the_reference_format(cli, oracle):
    r = _run("solve", "8", "--layers")
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().split("\n")
    head = dict(kv.split("=") for kv in lines[0].split())
    o = oracle.contract(8)
    assert head["N"] == "8" and head["Q(N)"] == "92" and head["verified"] == "true"
    assert int(head["peak_states"]) == o["peak_states"]
    assert (head["tensor_entries_examined"], head["tensor_entries_matched"]) == ("17", "17")
    assert int(head["row_operator_candidates"]) == o["row_operator_candidates"]
    assert int(head["row_operator_matched"]) == o["row_operator_matched"]
    assert set(head) == {"N", "Q(N)", "elapsed_s", "peak_rss_bytes", "peak_states", "tensor_entries_examined",
                         "tensor_entries_matched", "row_operator_candidates", "row_operator_matched", "verified"}
    assert lines[1] == ("row,input_states,tensor_entries_examined,tensor_entries_matched,row_operator_candidates,"
                        "row_operator_matched,completed_row_terms,output_states,output_weight,elapsed_s,"
                        "peak_rss_bytes")
    for line, l in zip(lines[2:], o["layers"]):
        f = line.split(",")
        assert int(f[0]) == l["row"] + 1
        assert [int(x) for x in f[1:9]] == [l["input_states"], l["tensor_entries_examined"],
                                            l["tensor_entries_matched"], l["row_operator_candidates"],
                                            l["row_operator_matched"], l["completed_row_terms"],
                                            l["output_states"], l["output_weight"]]
    assert len(lines) == 2 + 8


@pytest.mark.gpu
def test_bench_csv(cli, oracle):
    r = _run("bench", "10", "--min", "8", "--repeats", "2", "--csv")
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().split("\n")
    assert lines[0].startswith("N,count,known_count,verified,median_elapsed_s,min_elapsed_s,peak_rss_bytes")
    rows = [l.split(",") for l in lines[1:]]
    assert [int(r[0]) for r in rows] == [8, 9, 10]
    assert [int(r[1]) for r in rows] == [92, 352, 724]
    assert all(r[3] == "true" and r[-1] == "2" for r in rows)
    r = _run("bench", "6", "--min", "4", "--repeats", "1")
    assert r.returncode == 0 and r.stdout.count("verified=true") == 3
