"""Explicit-C generic site frontier on the GPU (contract_explicit_c_frontier,
src/lib.rs:961-967, 1519-1711) against the reference's published counters
(benchmarks/e34_corner_frontier_release.csv via the golden fixture) and the
CPU oracle."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

ORDERS = {"RowMajor": 0, "TopLeftDiamond": 1}
FIELDS = ("count", "peak_states", "peak_open_bonds", "tensor_entries_examined", "tensor_entries_accepted",
          "contracted_sites", "complete")


@pytest.mark.parametrize("order", [0, 1])
def test_small_boards_match_known_counts(ctx, qp, order):
    for n in range(0, 7):
        r = ctx.explicit_frontier(n, order, 5_000_000)
        assert r["complete"] and r["count"] == qp.known_count(n) and r["contracted_sites"] == n * n


@pytest.mark.parametrize("order_name", ["RowMajor", "TopLeftDiamond"])
@pytest.mark.parametrize("n", [7, 8, 9, 10, 11, 12])
def test_matches_published_counters(ctx, golden, order_name, n):
    want = golden["explicit_frontier"][order_name][str(n)]
    r = ctx.explicit_frontier(n, ORDERS[order_name], want["support_limit"])
    assert r["complete"] == want["complete"]
    assert r["count"] == want["count"]
    assert r["peak_states"] == want["peak_support"]
    assert r["peak_open_bonds"] == want["peak_open_bonds"]
    assert r["tensor_entries_examined"] == want["tensor_entries_examined"]
    assert r["tensor_entries_accepted"] == want["tensor_entries_accepted"]
    assert r["contracted_sites"] == want["contracted_sites"]


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8])
def test_every_field_matches_the_oracle(ctx, oracle, n, order):
    g = ctx.explicit_frontier(n, order)
    o = oracle.explicit_frontier(n, order)
    assert {k: g[k] for k in FIELDS} == {k: o[k] for k in FIELDS}


@pytest.mark.parametrize("order", [0, 1])
def test_support_limit_stops_at_the_same_site(ctx, oracle, order):
    for limit in (50, 500, 3000):  # below the peak support of both orders (3742, 9091)
        g = ctx.explicit_frontier(9, order, limit)
        o = oracle.explicit_frontier(9, order, limit)
        assert not g["complete"] and g["count"] is None
        assert g["peak_states"] == o["peak_states"] == limit + 1
        assert g["contracted_sites"] == o["contracted_sites"]
        assert g["peak_open_bonds"] == o["peak_open_bonds"]


def test_range_and_argument_errors(ctx, qp):
    with pytest.raises(qp.ContractionError) as e:
        ctx.explicit_frontier(22, 0, 10)
    assert e.value.code == qp.QPEPS_ERR_RANGE and "N <= 21" in e.value.message
    with pytest.raises(qp.ContractionError) as e:
        ctx.explicit_frontier(5, 0, 0)
    assert e.value.code == qp.QPEPS_ERR_INVALID and "support limit must be positive" in e.value.message


@pytest.mark.parametrize("order", [0, 1])
def test_partitioned_merge_equals_global_table(qp, order):
    """The explicit-C frontier through the 128-bit partitions (the default)
    and through the global table (merge_auto = MERGE_HASH) agree on every
    field, complete and stopped at a support limit. After its first step a
    partitioned run launches a scatter and a merge per site (its merges count
    the next step's matches), so it launches at most one kernel more than the
    table's expand-insert and compaction."""
    part, table = qp.Context(0), qp.Context(0)
    try:
        table.set_tuning(merge_auto=qp.MERGE_HASH)
        for n in range(1, 13):
            a, b = part.explicit_frontier(n, order), table.explicit_frontier(n, order)
            assert {k: a[k] for k in FIELDS} == {k: b[k] for k in FIELDS}, n
            assert a["merge"] == qp.MERGE_PARTITION and b["merge"] == qp.MERGE_HASH
            assert a["gpu_launches"] <= b["gpu_launches"] + 1
        for limit in (50, 3000, 200_000):
            a, b = part.explicit_frontier(11, order, limit), table.explicit_frontier(11, order, limit)
            assert {k: a[k] for k in FIELDS} == {k: b[k] for k in FIELDS}, limit
    finally:
        part.close()
        table.close()


def test_partition_overflow_retries_exactly(qp, golden):
    """At fill 0.95 partitions of 1024 slots overflow on large steps; the
    merge then writes nothing and the step is retried with smaller
    partitions, so the published counters still hold."""
    c = qp.Context(0)
    try:
        c.set_tuning(partition_fill=0.95)
        for name, order in ORDERS.items():
            want = golden["explicit_frontier"][name]["12"]
            r = c.explicit_frontier(12, order, want["support_limit"])
            assert r["count"] == want["count"] and r["peak_states"] == want["peak_support"]
            assert r["tensor_entries_accepted"] == want["tensor_entries_accepted"]
    finally:
        c.close()
