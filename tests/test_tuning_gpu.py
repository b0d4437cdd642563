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
    combo for combo in itertools.product((0, 1, 2, 3, 4), (2, 4), (0, 1), (0, 1, 3), (0, 1, 2)) if combo[2] == 1 or combo[4] == 0
])
@pytest.mark.parametrize("compact", [0, 1])
def test_every_kernel_shape_matches_oracle(tctx, oracle, scatter, ppl, merge, wide, fold, compact):
    tctx.set_tuning(scatter_kind=scatter, parents_per_lane=ppl, merge_kind=merge, wide_merge=wide,
                    fold_weights=fold, merge_compact=compact)
    for n in (9, 13):
        got = tctx.contract_rows(n)
        want = _oracle(oracle, n)
        assert got.count == want["count"]
        assert got.peak_states == want["peak_states"]
        assert [l.output_states for l in got.layers] == [l["output_states"] for l in want["layers"]]


@pytest.mark.parametrize("n", [14, 16, 17])
def test_class_scatter_equals_the_window_scatter(tctx, qp, n):
    # Class-grouped partitions: other partitions, the same merged boundary,
    # so the same counts and per-row metrics, eagerly and under graph replay.
    ref = tctx.contract_rows(n)
    tctx.set_tuning(scatter_kind=qp.SCATTER_CLASS)
    got = tctx.contract_rows(n)
    assert got.count == ref.count == qp.known_count(n)
    assert _layers(got) == _layers(ref)
    assert got.peak_states == ref.peak_states
    # Not graph-captured: repeated contractions run eagerly, exact each time.
    first = tctx.contract_rows(n, use_graph=1)
    again = tctx.contract_rows(n, use_graph=1)
    assert again.device["gpu_launches"] == first.device["gpu_launches"]
    assert first.count == again.count == ref.count
    assert _layers(again) == _layers(ref)


def test_class_scatter_undersized_plan_retries_exactly(tctx, qp, oracle):
    # A coarse sample (1 parent in 64) with small planned partitions makes the
    # plan's estimates noisy; a partition that overflows makes the merge write
    # nothing and the row runs again with more partitions.
    tctx.set_tuning(scatter_kind=qp.SCATTER_CLASS, unit_sample=64, unit_target=1800)
    for n in (12, 15):
        got = tctx.contract_rows(n)
        assert got.count == qp.known_count(n)
        if n <= 12:
            want = _oracle(oracle, n)
            assert [l.output_states for l in got.layers] == [l["output_states"] for l in want["layers"]]


@pytest.mark.parametrize("R", [1, 2])
def test_class_scatter_residue_planes_prefixes_and_budget(tctx, qp, oracle, R):
    tctx.set_tuning(scatter_kind=qp.SCATTER_CLASS, fold_weights=0)
    n = 12
    got = tctx.contract_rows(n, residues=R)
    want = _oracle(oracle, n)
    assert got.count == want["count"]
    assert [(l.output_states, l.output_weight) for l in got.layers] == [
        (l["output_states"], l["output_weight"]) for l in want["layers"]]
    for prefix in ([3], [1, 4], [0, 2, 5]):
        assert tctx.count(13, prefix) == oracle.contract(13, symmetry=False, prefix=prefix)["count"]
    small = tctx.contract_rows(14, device_budget_bytes=16 << 20)
    assert small.count == qp.known_count(14) and small.device["batches"] > 1


@pytest.mark.parametrize("n", [15, 16, 17])
def test_two_level_scatter_equals_the_window_scatter(tctx, qp, n):
    # Coarse buckets then partitions, each written as ordered runs: the same
    # partitions, so the same boundary, counts and per-row metrics.
    ref = tctx.contract_rows(n)
    tctx.set_tuning(scatter_kind=qp.SCATTER_TWO_LEVEL)
    got = tctx.contract_rows(n)
    assert got.count == ref.count == qp.known_count(n)
    assert _layers(got) == _layers(ref)
    assert got.peak_states == ref.peak_states
    first = tctx.contract_rows(n, use_graph=1)
    replay = tctx.contract_rows(n, use_graph=1)
    assert first.count == replay.count == qp.known_count(n)
    assert _layers(replay) == _layers(ref)


def test_two_level_scatter_residues_budgets_and_prefixes(tctx, qp, oracle):
    tctx.set_tuning(scatter_kind=qp.SCATTER_TWO_LEVEL)
    # One residue plane (N <= 12) and exact weights use 16-byte candidates;
    # three or four planes (32-byte candidates) keep the window scatter.
    for residues in (1, 2):
        assert tctx.contract_rows(12, residues=residues).count == qp.known_count(12)
    tctx.set_tuning(fold_weights=0)
    for residues in (2, 3, 4):
        assert tctx.contract_rows(12, residues=residues).count == qp.known_count(12)
    tctx.set_tuning(fold_weights=2, partition_fill=0.3, spread_cursors_below=0)
    assert tctx.contract_rows(14, device_budget_bytes=8 << 20).count == qp.known_count(14)
    for n, prefix in [(14, [3, 0]), (15, [7, 2, 4])]:
        want = oracle.contract(n, symmetry=False, prefix=prefix)["count"]
        assert tctx.count(n, prefix) == want


def test_low_partition_fill_and_slice_margin_are_exact(tctx, qp):
    ref = tctx.contract_rows(15)
    tctx.set_tuning(partition_fill=0.3, spread_cursors_below=0, wide_above_parts=1)
    got = tctx.contract_rows(15)
    assert got.count == qp.known_count(15)
    assert _layers(got) == _layers(ref)
    tctx.set_tuning(slice_margin=8.0)
    assert tctx.contract_rows(12, device_budget_bytes=4 << 20).count == qp.known_count(12)


@pytest.mark.parametrize("field,value", [
    ("scatter_kind", 5), ("parents_per_lane", 3), ("merge_kind", 5), ("wide_merge", 4), ("batch_lanes", 0),
    ("merge_compact", 2), ("unit_target", 100), ("unit_sample", 3), ("scatter_block", 300), ("merge_auto", 0),
    ("slice_rows", 5),
    ("partition_fill", 0.99), ("partition_fill", 0.1), ("slice_margin", 0.5), ("fold_weights", 3),
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
    assert t["scatter_kind"] in (0, 1, 2, 4) and t["parents_per_lane"] in (2, 4) and t["merge_kind"] in (0, 1)
    assert t["scatter_block"] in (128, 256, 512) and t["batch_lanes"] in (1, 2) and t["slice_rows"] in (1, 2)
    assert t["merge_auto"] in (qp.MERGE_PARTITION, qp.MERGE_HASH)
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


@pytest.mark.parametrize("block", [128, 512])
def test_scatter_block_sizes_match_oracle(tctx, qp, oracle, block):
    for kind in (0, 1, 4):
        tctx.set_tuning(scatter_block=block, scatter_kind=kind)
        for n in (9, 13):
            got = tctx.contract_rows(n)
            want = _oracle(oracle, n)
            assert got.count == want["count"]
            assert [l.output_states for l in got.layers] == [l["output_states"] for l in want["layers"]]


def test_merge_auto_and_slice_rows_are_exact(tctx, qp, oracle):
    tctx.set_tuning(merge_auto=qp.MERGE_HASH)
    r = tctx.contract_rows(11)
    assert r.device["merge"] == qp.MERGE_HASH and r.count == qp.known_count(11)
    tctx.set_tuning(merge_auto=qp.MERGE_PARTITION, slice_rows=2)
    r = tctx.contract_rows(13)
    want = _oracle(oracle, 13)
    assert r.device["merge"] == qp.MERGE_PARTITION and r.count == want["count"]
    assert r.device["slice_depth"] >= 2
    assert [l.output_states for l in r.layers] == [l["output_states"] for l in want["layers"]]


def test_autotune_rejects_probe_sizes_outside_range(tctx, qp):
    with pytest.raises(qp.ContractionError) as e:
        tctx.autotune(n=20, repeats=1)
    assert e.value.code == qp.QPEPS_ERR_RANGE


@pytest.mark.parametrize("n", [13, 16, 17])
def test_folded_exact_and_residue_accumulators_agree(tctx, qp, n):
    runs = []
    for fold in (0, 1, 2):
        tctx.set_tuning(fold_weights=fold)
        runs.append(tctx.contract_rows(n))
    assert all(r.count == qp.known_count(n) for r in runs)
    assert _layers(runs[0]) == _layers(runs[1]) == _layers(runs[2])
    assert runs[0].device["count_residues"] == runs[1].device["count_residues"] == runs[2].device["count_residues"]


def test_exact_weights_survive_spills_and_prefixes(tctx, qp, oracle):
    tctx.set_tuning(fold_weights=2)
    # a budget that splits the live boundary to the host and back
    assert tctx.contract_rows(14, device_budget_bytes=6 << 20).count == qp.known_count(14)
    for prefix in ([5], [2, 9], [0, 7, 3]):
        assert tctx.count(16, prefix) == oracle.contract(16, backend=oracle.PARALLEL_SORT_REDUCE, threads=8,
                                                         symmetry=False, prefix=prefix)["count"]


def test_fold_and_exact_weights_at_the_n20_bound(tctx, qp):
    # Boards with up to 20 free rows use the one-plane accumulators: an N=20
    # prefix slice, and an N=21 slice with one row placed (free rows 20).
    got = []
    for fold in (0, 1, 2):
        tctx.set_tuning(fold_weights=fold)
        got.append(tctx.count_with_stats(20, [3, 0, 7, 11]))
    assert got[0][0] == got[1][0] == got[2][0]
    got = []
    for fold in (0, 2):
        tctx.set_tuning(fold_weights=fold)
        got.append(tctx.count_with_stats(21, [10, 3, 0, 8, 16]))
    assert got[0][0] == got[1][0]
    assert got[1][1].device["residues"] == 2
