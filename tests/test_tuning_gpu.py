"""Tuning knobs and the autotuner (no reference counterpart): every tuning
gives the oracle's counts and per-row metrics; only speed changes."""
from __future__ import annotations

import itertools
import json

import pytest

pytestmark = pytest.mark.gpu

LAYER_FIELDS = ("input_states", "output_states", "completed_row_terms", "output_weight",
                "row_operator_candidates", "row_operator_matched")


def _layers(r):
    return [tuple(getattr(l, f) for f in LAYER_FIELDS) for l in r.layers]


_ORACLE = {}


def _oracle(oracle, n):
    if n not in _ORACLE:
        _ORACLE[n] = oracle.contract(n)
    return _ORACLE[n]


@pytest.fixture()
def tctx(qp):
    c = qp.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("scatter,ppl,merge,wide,fold", [
    combo for combo in itertools.product((0, 1), (2, 4), (0, 1), (0, 1), (0, 1)) if combo[2] == 1 or combo[4] == 0
])
def test_every_kernel_shape_matches_oracle(tctx, oracle, scatter, ppl, merge, wide, fold):
    tctx.set_tuning(scatter_kind=scatter, parents_per_lane=ppl, merge_kind=merge, wide_merge=wide,
                    fold_weights=fold)
    for n in (9, 13):
        got = tctx.contract_rows(n)
        want = _oracle(oracle, n)
        assert got.count == want["count"]
        assert got.peak_states == want["peak_states"]
        assert [l.output_states for l in got.layers] == [l["output_states"] for l in want["layers"]]


def test_low_partition_fill_and_slice_margin_are_exact(tctx, qp):
    ref = tctx.contract_rows(15)
    tctx.set_tuning(partition_fill=0.3, spread_cursors_below=0, wide_above_parts=1)
    got = tctx.contract_rows(15)
    assert got.count == qp.known_count(15)
    assert _layers(got) == _layers(ref)
    tctx.set_tuning(slice_margin=8.0)
    assert tctx.contract_rows(12, device_budget_bytes=4 << 20).count == qp.known_count(12)


@pytest.mark.parametrize("field,value", [
    ("scatter_kind", 2), ("parents_per_lane", 3), ("merge_kind", 5), ("wide_merge", 3),
    ("partition_fill", 0.99), ("partition_fill", 0.1), ("slice_margin", 0.5), ("fold_weights", 2),
])
def test_out_of_range_tuning_is_rejected_and_kept(tctx, qp, field, value):
    before = tctx.tuning
    with pytest.raises(qp.ContractionError) as e:
        tctx.set_tuning(**{field: value})
    assert e.value.code == qp.QPEPS_ERR_INVALID
    assert tctx.tuning == before


def test_get_tuning_reflects_set(tctx):
    t = tctx.set_tuning(parents_per_lane=2, merge_kind=0, partition_fill=0.7)
    assert t["parents_per_lane"] == 2 and t["merge_kind"] == 0 and abs(t["partition_fill"] - 0.7) < 1e-12


def test_autotune_picks_a_grid_point_and_caches_it(tctx, qp, tmp_path):
    cache = tmp_path / "tuning.json"
    out = tctx.autotune(n=12, repeats=1, cache=cache)
    assert not out["cached"] and out["device_ms"] > 0
    t = out["tuning"]
    assert t["scatter_kind"] in (0, 1) and t["parents_per_lane"] in (2, 4) and t["merge_kind"] in (0, 1)
    assert tctx.tuning["scatter_kind"] == t["scatter_kind"]
    entries = json.loads(cache.read_text())
    assert len(entries) == 1 and next(iter(entries)).endswith("|n=12")
    other = qp.Context(0)
    try:
        again = other.autotune(n=12, repeats=1, cache=cache)
        assert again["cached"] and again["tuning"] == t
        assert other.contract_rows(14).count == qp.known_count(14)
    finally:
        other.close()


def test_autotune_rejects_probe_sizes_outside_range(tctx, qp):
    with pytest.raises(qp.ContractionError) as e:
        tctx.autotune(n=19, repeats=1)
    assert e.value.code == qp.QPEPS_ERR_RANGE


@pytest.mark.parametrize("n", [13, 16, 17])
def test_folded_and_residue_accumulators_agree(tctx, qp, n):
    tctx.set_tuning(fold_weights=0)
    a = tctx.contract_rows(n)
    tctx.set_tuning(fold_weights=1)
    b = tctx.contract_rows(n)
    assert a.count == b.count == qp.known_count(n)
    assert _layers(a) == _layers(b)
    assert a.device["count_residues"] == b.device["count_residues"]


def test_fold_is_exact_at_n20_bound(tctx, qp):
    # 20! < p0 * p1: the largest board that folds; its row weights must match
    # the residue accumulator's on a prefix slice that runs in seconds.
    tctx.set_tuning(fold_weights=0)
    a = tctx.count_with_stats(20, [3, 0, 7, 11])
    tctx.set_tuning(fold_weights=1)
    b = tctx.count_with_stats(20, [3, 0, 7, 11])
    assert a[0] == b[0]
    assert a[1].device["residues"] == b[1].device["residues"] == 2
