"""The C-ABI library loads and exports every symbol include/qpeps.h declares.

CPU only: no call here launches device work. Host-only entry points
(version, known counts, options, C certification) are exercised directly.
"""
from __future__ import annotations

import re
import subprocess

import pytest

from conftest import ROOT


def _declared_functions():
    text = (ROOT / "include" / "qpeps.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qpeps_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = _declared_functions()
    for required in ["qpeps_contract_rows", "qpeps_count", "qpeps_count_batch", "qpeps_known_count",
                     "qpeps_ctx_create", "qpeps_ctx_destroy", "qpeps_version", "qpeps_certify_c"]:
        assert required in names


def test_library_exports_every_declared_symbol(qp):
    out = subprocess.run(["nm", "-D", "--defined-only", str(qp.LIBRARY_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (qpeps_[a-z0-9_]+)$", out, flags=re.M))
    missing = [n for n in _declared_functions() if n not in exported]
    assert not missing, missing
    lib = qp.library()
    for n in _declared_functions():
        getattr(lib, n)


def test_version_and_known_counts(qp, golden):
    assert "sm_103a" in qp.version()
    assert [qp.known_count(n) for n in range(28)] == [int(v) for v in golden["known_count"]]
    assert qp.known_count(28) is None


def test_options_default_matches_reference_semantics(qp):
    o = qp.options()
    assert o.granularity == qp.GRAIN_ROW and o.symmetry == 1 and o.collect_layers == 1


def test_certify_c_accepts_sec_vi_and_fails_closed(qp, oracle):
    c = oracle.c_entries()
    qp.certify_c(c)
    cases = {
        "unit Sec. VI coefficients": [(l, 2 if i == 0 else v) for i, (l, v) in enumerate(c)],
        "missing a pass-through": c[1:],
        "missing the occupied entry": [e for e in c if e[0] != 0b10101010],
        "multiple occupied": c + [(0b10101010, 1)],
        "outside the Sec. VI row automaton": c + [(0b00000010, 1)],
        "duplicate C pass-through": c + [(0, 1)],
    }
    for msg, table in cases.items():
        with pytest.raises(qp.ContractionError, match=msg) as ei:
            qp.certify_c(table)
        assert ei.value.code == qp.QPEPS_ERR_INVALID
        assert oracle.compile_check(table) is not None


def test_tuning_default_is_the_library_default(qp):
    t = qp.tuning_default()
    assert t["scatter_kind"] == qp.SCATTER_WINDOW
    assert t["merge_kind"] == qp.MERGEK_CLAIM
    assert t["parents_per_lane"] in (2, 4)
    assert t["wide_merge"] == 2
    assert 0.3 <= t["partition_fill"] <= 0.95
    assert t["slice_margin"] >= 1.0


def test_no_host_fallback_without_a_device(qp):
    # The library computes only on the GPU: without a CUDA device, creating a
    # context (and so any contraction) fails with QPEPS_ERR_CUDA instead of
    # running on the host.
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(qp.ContractionError) as e:
        qp.Context(0)
    assert e.value.code == qp.QPEPS_ERR_CUDA
    with pytest.raises(qp.ContractionError):
        qp.contract_rows(8)


def test_shipped_tuning_cache_matches_this_library(qp):
    """Every entry of the GB300 tuning cache is keyed by this library's
    version and names only fields of qpeps_tuning, within their ranges."""
    import json

    entries = json.loads((qp.LIBRARY_PATH.parent / "tuning_gb300.json").read_text())
    fields = {name for name, _ in qp.Tuning._fields_} - {"struct_size", "reserved"}
    assert entries
    for key, e in entries.items():
        device, ver, probe = key.split("|")
        assert device == "NVIDIA GB300" and ver == qp.version() and probe.startswith("n=")
        t = e["tuning"]
        assert set(t) <= fields and e["device_ms"] > 0
        assert 0.3 <= t["partition_fill"] <= 0.95 and 1 <= t["batch_lanes"] <= 8 and 1.0 <= t["slice_margin"] <= 64
        assert t["scatter_kind"] in (0, 1, 2, 4)  # the class-grouped scatter is never cached
