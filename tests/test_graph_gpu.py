"""CUDA-graph replay of repeated contractions (qpeps_options.use_graph): the
second identical contraction on a context replays the captured row steps as
one graph and must return exactly the eager run's count and metrics."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("input_states", "output_states", "completed_row_terms", "output_weight", "row_operator_candidates",
          "row_operator_matched")


def _metrics(r):
    return (r.count, r.peak_states, r.row_operator_candidates, r.row_operator_matched,
            [tuple(getattr(l, f) for f in FIELDS) for l in r.layers])


@pytest.fixture()
def gctx(qp):
    c = qp.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("n", [6, 11, 14, 16])
def test_replay_equals_eager(gctx, qp, n):
    eager = gctx.contract_rows(n, use_graph=1)
    replay = gctx.contract_rows(n, use_graph=1)
    again = gctx.contract_rows(n, use_graph=1)
    assert eager.count == qp.known_count(n)
    assert _metrics(replay) == _metrics(eager) == _metrics(again)
    rows = sum(1 for l in eager.layers if l.input_states) or 1
    if n >= 11:
        # replay: scatter + merge per device row, no per-row count launch
        assert replay.device["gpu_launches"] < eager.device["gpu_launches"]
        assert replay.device["gpu_launches"] <= 2 * rows


def test_replay_of_several_device_batches(gctx, qp):
    budget = 48 << 20  # forces predictive slicing into several device batches
    eager = gctx.contract_rows(15, use_graph=1, device_budget_bytes=budget)
    replay = gctx.contract_rows(15, use_graph=1, device_budget_bytes=budget)
    assert eager.count == replay.count == qp.known_count(15)
    assert _metrics(replay) == _metrics(eager)


def test_prefix_requests_replay_per_prefix(gctx, oracle):
    a1 = gctx.count_with_stats(13, [2, 5], use_graph=1)
    a2 = gctx.count_with_stats(13, [2, 5], use_graph=1)
    b = gctx.count_with_stats(13, [4, 1], use_graph=1)   # different prefix: no replay of the first graph
    assert a1[0] == a2[0] == oracle.contract(13, symmetry=False, prefix=[2, 5])["count"]
    assert b[0] == oracle.contract(13, symmetry=False, prefix=[4, 1])["count"]


def test_other_options_or_tuning_do_not_replay(gctx, qp):
    first = gctx.contract_rows(14, use_graph=1)
    gctx.set_tuning(merge_kind=0)
    second = gctx.contract_rows(14, use_graph=1)       # new tuning: eager again
    assert second.device["gpu_launches"] == first.device["gpu_launches"]
    third = gctx.contract_rows(14, use_graph=1, collect_layers=0)
    assert first.count == second.count == third.count == qp.known_count(14)


def test_eager_run_between_replays_keeps_results_exact(gctx, qp):
    gctx.contract_rows(14, use_graph=1)
    gctx.contract_rows(15)                               # grows the context's buffers
    r = gctx.contract_rows(14, use_graph=1)
    assert r.count == qp.known_count(14)


@pytest.mark.parametrize("lanes", [1, 2, 3])
def test_concurrent_batch_lanes_replay_exactly(gctx, qp, lanes):
    # Device batches are independent sub-contractions: the replay runs them on
    # `batch_lanes` streams with a buffer set each; every row's metrics and
    # the count equal the eager run's, whichever lane ran which batch.
    gctx.set_tuning(batch_lanes=lanes)
    budget = 48 << 20  # several device batches
    eager = gctx.contract_rows(15, use_graph=1, device_budget_bytes=budget)
    assert eager.device["batches"] > 1
    replay = gctx.contract_rows(15, use_graph=1, device_budget_bytes=budget)
    again = gctx.contract_rows(15, use_graph=1, device_budget_bytes=budget)
    assert replay.device["gpu_launches"] < eager.device["gpu_launches"]  # replayed
    assert eager.count == replay.count == again.count == qp.known_count(15)
    assert _metrics(replay) == _metrics(eager) == _metrics(again)


def test_class_partitions_are_not_captured(gctx, qp):
    # Class-grouped partitions run eagerly even with use_graph (they are not
    # captured); repeated contractions stay exact.
    gctx.set_tuning(batch_lanes=2, scatter_kind=qp.SCATTER_CLASS)
    budget = 48 << 20
    eager = gctx.contract_rows(15, use_graph=1, device_budget_bytes=budget)
    again = gctx.contract_rows(15, use_graph=1, device_budget_bytes=budget)
    assert again.device["gpu_launches"] == eager.device["gpu_launches"]
    assert eager.count == again.count == qp.known_count(15)
    assert _metrics(again) == _metrics(eager)
