"""bench.py's reference arm on the CPU: one JSON line with the keys the
benchmark contract names, and silence on every rank but 0.

The reference arm times the oracle's threaded restatement of the reference's
sort-reduce driver on a bounded sample (the first rows of Q(N)); a small N
keeps this test to seconds.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

from conftest import ROOT


def _bench(*args, env=None):
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                          timeout=300, cwd=str(ROOT), env=env)


def test_reference_arm_prints_one_contract_line(oracle):
    r = _bench("--impl", "reference", "--n", "10", "--cpu-rows", "6", "--steps", "2", "--warmup", "3")
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["steps"] == 2 and line["warmup"] == 3 and line["higher_is_better"] is True
    assert line["value"] > 0 and line["unit"] == "boundary entries/s"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "first 6 rows of Q(10)" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["n"] == 10 and "workload" in line["config"]


def test_reference_arm_is_silent_on_other_ranks(oracle):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = _bench("--impl", "reference", "--n", "10", "--cpu-rows", "6", "--steps", "1", "--warmup", "3", env=env)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
