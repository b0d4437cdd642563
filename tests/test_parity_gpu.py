"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Bar: bit-exact. Counts, peak support, work counters and every per-row
(input_states, row_operator_candidates, row_operator_matched,
completed_row_terms, output_states, output_weight) equal the oracle's
restatement of contract_rows (src/lib.rs:5287-5415) and the reference's
published golden values.
"""
from __future__ import annotations

import math
import random

import pytest

import oracle_py as O

pytestmark = pytest.mark.gpu

LAYER_FIELDS = ["row", "input_states", "row_operator_candidates", "row_operator_matched", "completed_row_terms",
                "output_states", "output_weight"]


def _gpu_layers(r):
    return [tuple(getattr(l, f) for f in LAYER_FIELDS) for l in r.layers]


def _oracle_layers(o):
    return [tuple(l[f] for f in LAYER_FIELDS) for l in o["layers"]]


@pytest.mark.parametrize("n", range(0, 13))
def test_contract_rows_matches_oracle_row_by_row(ctx, oracle, n):
    g = ctx.contract_rows(n)
    o = oracle.contract(n, backend=O.SORT_REDUCE)
    assert g.count == o["count"] == oracle.known_count(n)
    assert g.peak_states == o["peak_states"]
    assert g.row_operator_candidates == o["row_operator_candidates"]
    assert g.row_operator_matched == o["row_operator_matched"]
    assert (g.tensor_entries_examined, g.tensor_entries_matched) == (o["tensor_entries_examined"],
                                                                    o["tensor_entries_matched"])
    assert _gpu_layers(g) == _oracle_layers(o)


@pytest.mark.parametrize("n", [13, 14])
def test_orbit_path_matches_published_layers(ctx, golden, n):
    g = ctx.contract_rows(n)
    e12 = golden["e12_summary"]["d4_orbit_serial_sort_reduce"][str(n)]
    assert g.count == e12["count"]
    assert g.peak_states == e12["peak_support"]
    assert g.row_operator_candidates == e12["row_operator_candidates"]
    assert g.row_operator_matched == e12["row_operator_matched"]
    assert [1] + [l.output_states for l in g.layers] == golden["orbit_layers_output_states"][str(n)]


def test_n16_matches_published_peak_and_matched_work(ctx, golden):
    # benchmarks/e36_joint_u64_release.csv, N=16 (orbit path)
    g = ctx.contract_rows(16)
    ref = golden["e36_orbit_n16"]["16"]
    assert g.count == ref["count"] == 14772512
    assert g.peak_states == ref["peak_support"]
    assert g.row_operator_matched == ref["row_operator_matched"]
    assert g.device["residues"] == 2 and g.device["key_bits"] == 64


@pytest.mark.parametrize("n", range(1, 12))
def test_dense_no_symmetry_matches_oracle(ctx, oracle, n):
    g = ctx.contract_rows(n, symmetry=0)
    o = oracle.contract(n, backend=O.SORT_REDUCE, symmetry=False)
    assert g.count == o["count"]
    assert g.peak_states == o["peak_states"]
    assert _gpu_layers(g) == _oracle_layers(o)


def test_dense_peaks_match_published(ctx, golden):
    for n in [10, 12, 14]:
        g = ctx.contract_rows(n, symmetry=0)
        assert g.peak_states == golden["naive_dense_hashmap"][str(n)]["peak_support"]
        assert g.count == golden["naive_dense_hashmap"][str(n)]["count"]


@pytest.mark.parametrize("n", range(1, 11))
def test_site_grain_equals_row_grain(ctx, n):
    # One plain launch per site applying the explicit C table.
    s = ctx.contract_rows(n, granularity=1)
    r = ctx.contract_rows(n)
    assert s.count == r.count
    assert s.peak_states >= r.peak_states
    assert [(l.input_states, l.output_states, l.output_weight, l.completed_row_terms) for l in s.layers] == [
        (l.input_states, l.output_states, l.output_weight, l.completed_row_terms) for l in r.layers]


SITEWISE_FIELDS = ["row", "input_states", "tensor_entries_examined", "tensor_entries_matched",
                   "row_operator_candidates", "row_operator_matched", "completed_row_terms", "output_states",
                   "output_weight"]


@pytest.mark.parametrize("n", range(1, 11))
def test_site_grain_counters_match_sitewise_backend(ctx, oracle, n):
    # The plain per-site form is the reference's sitewise backend
    # (contract_rows_with_backend(Sitewise), src/lib.rs:5633-5750): per row the
    # C entries its per-parent site kernel matched (src/lib.rs:538-541), no
    # row-operator counts, and the same frontier, against the oracle's HashMap
    # sitewise driver on the dense (no symmetry) board.
    g = ctx.contract_rows(n, granularity=1, symmetry=0)
    o = oracle.contract(n, backend=O.HASH_SITEWISE, symmetry=False)
    assert g.count == o["count"] == oracle.known_count(n)
    assert [tuple(getattr(l, f) for f in SITEWISE_FIELDS) for l in g.layers] == [
        tuple(l[f] for f in SITEWISE_FIELDS) for l in o["layers"]]
    assert (g.tensor_entries_examined, g.tensor_entries_matched) == (o["tensor_entries_examined"],
                                                                    o["tensor_entries_matched"])
    assert (g.row_operator_candidates, g.row_operator_matched) == (0, 0) == (o["row_operator_candidates"],
                                                                             o["row_operator_matched"])
    assert g.peak_states == o["peak_states"]


def test_site_grain_n16_plain_form(ctx, qp, golden):
    # Config 2: one plain launch per site over the whole N=16 board; every row
    # equals the batched row form (whose N=16 peak and matched work equal the
    # published benchmarks/e36_joint_u64_release.csv values).
    s = ctx.contract_rows(16, granularity=1)
    r = ctx.contract_rows(16)
    assert s.count == r.count == 14772512 == golden["e36_orbit_n16"]["16"]["count"]
    assert s.device["merge"] == qp.MERGE_HASH
    assert [(l.input_states, l.completed_row_terms, l.output_states, l.output_weight) for l in s.layers] == [
        (l.input_states, l.completed_row_terms, l.output_states, l.output_weight) for l in r.layers]
    assert max(l.output_states for l in r.layers) == golden["e36_orbit_n16"]["16"]["peak_support"]
    # 16 x 16 site launches plus the row counts, against 2 or 3 launches per row
    assert s.device["gpu_launches"] > 16 * 15 and r.device["gpu_launches"] < 3 * 16


@pytest.mark.parametrize("n", [1, 4, 8, 11, 12])
def test_forced_wide_keys_are_exact(ctx, oracle, n):
    g = ctx.contract_rows(n, key_bits=128)
    o = oracle.contract(n)
    assert g.device["key_bits"] == 128
    assert g.count == o["count"]
    assert _gpu_layers(g) == _oracle_layers(o)
    s = ctx.contract_rows(n, key_bits=128, granularity=1)
    assert s.count == o["count"]


def _legal_prefix(n, k, seed):
    import random

    rng = random.Random(seed)
    while True:
        cols, ok = [], True
        for r in range(k):
            free = [c for c in range(n) if all(c != q and abs(c - q) != r - i for i, q in enumerate(cols))]
            if not free:
                ok = False
                break
            cols.append(rng.choice(free))
        if ok:
            return cols


@pytest.mark.parametrize("n,k", [(22, 7), (23, 8), (24, 9), (26, 11), (28, 13), (30, 15), (42, 30)])
def test_wide_boards_match_oracle(ctx, oracle, n, k):
    # N = 22: the 3N - 2 live bits of a row key fill a u64 exactly (compact
    # layout); N >= 23 needs u128 keys (natural, not forced), merged through
    # the partitioned merge with 128-bit keys. N = 42 is the widest board the
    # reference accepts. The prefixes keep the oracle's frontier at up to
    # about 0.4 M states.
    prefix = _legal_prefix(n, k, 1000 + n)
    count, res = ctx.count_with_stats(n, prefix)
    assert res.device["key_bits"] == (64 if n == 22 else 128)
    # residues certify (N - k)!: completions place N - k queens in distinct columns
    bound, prod, want_r = math.factorial(n - k), 1, 0
    for p in (2147483647, 2147483629, 2147483587, 2147483579):
        prod *= p
        want_r += 1
        if prod > bound:
            break
    assert res.device["residues"] == want_r
    want = oracle.contract(n, backend=oracle.PARALLEL_SORT_REDUCE, threads=8, symmetry=False, prefix=prefix)
    assert count == want["count"]
    assert res.peak_states == want["peak_states"]


@pytest.mark.parametrize("n", [13, 15, 16])
def test_wide_key_partitioned_merge_equals_global_table(ctx, qp, n):
    # 128-bit keys forced: the partitioned scatter and merge with 32-byte
    # candidates give the global table's frontier row by row, and the
    # default u64 path's; a CUDA-graph replay of it is exact too.
    part = ctx.contract_rows(n, key_bits=128, merge=qp.MERGE_PARTITION)
    table = ctx.contract_rows(n, key_bits=128, merge=qp.MERGE_HASH)
    narrow = ctx.contract_rows(n)
    assert part.device["merge"] == qp.MERGE_PARTITION and part.device["key_bits"] == 128
    assert part.count == table.count == narrow.count == qp.known_count(n)
    assert _gpu_layers(part) == _gpu_layers(table) == _gpu_layers(narrow)
    first = ctx.contract_rows(n, key_bits=128, use_graph=1)
    again = ctx.contract_rows(n, key_bits=128, use_graph=1)
    assert again.device["gpu_launches"] < first.device["gpu_launches"]
    assert _gpu_layers(again) == _gpu_layers(narrow) and again.count == narrow.count


@pytest.mark.parametrize("residues", [1, 3, 4])
def test_wide_key_partitioned_merge_residue_planes(ctx, oracle, residues):
    n = 11 if residues == 1 else 12
    g = ctx.contract_rows(n, key_bits=128, residues=residues)
    assert g.device["residues"] == residues and g.device["key_bits"] == 128
    assert g.count == oracle.known_count(n)
    assert _gpu_layers(g) == _oracle_layers(oracle.contract(n))


def test_wide_key_partitioned_merge_wide_boards_both_merges(ctx, qp, oracle):
    prefix = _legal_prefix(24, 10, 77)
    a = ctx.count(24, prefix, merge=qp.MERGE_PARTITION)
    b = ctx.count(24, prefix, merge=qp.MERGE_HASH)
    want = oracle.contract(24, backend=oracle.PARALLEL_SORT_REDUCE, threads=8, symmetry=False, prefix=prefix)
    assert a == b == want["count"]


@pytest.mark.parametrize("residues", [1, 2, 3, 4])
def test_forced_residue_planes_are_exact(ctx, oracle, residues):
    n = 10
    g = ctx.contract_rows(n, residues=residues)
    assert g.device["residues"] == residues
    assert g.count == 724
    assert _gpu_layers(g) == _oracle_layers(oracle.contract(n))


def test_too_few_residues_for_n_factorial_is_rejected(ctx, qp):
    with pytest.raises(qp.ContractionError) as ei:
        ctx.contract_rows(14, residues=1)
    assert ei.value.code == qp.QPEPS_ERR_RANGE


def test_rejects_virtual_boundaries_wider_than_u128_layout(ctx, qp):
    with pytest.raises(qp.ContractionError, match="supports N <= 42") as ei:
        ctx.contract_rows(43)
    assert ei.value.code == qp.QPEPS_ERR_RANGE


def test_empty_board(ctx):
    g = ctx.contract_rows(0)
    assert (g.count, g.peak_states, len(g.layers)) == (1, 1, 0)


def test_prefix_counts_match_oracle(ctx, oracle):
    rng = random.Random(20261203)
    for _ in range(60):
        n = rng.randint(4, 12)
        k = rng.randint(0, 3)
        prefix = [rng.randrange(n) for _ in range(k)]
        want = oracle.contract(n, symmetry=False, prefix=prefix)["count"] if k else oracle.known_count(n)
        assert ctx.count(n, prefix) == want, (n, prefix)


def test_prefix_sum_rule_at_n14(ctx, oracle):
    assert sum(ctx.count(14, [c]) for c in range(14)) == oracle.known_count(14)


def test_complete_prefix_counts_itself(ctx):
    assert ctx.count(8, [0, 4, 7, 5, 2, 6, 1, 3]) == 1
    assert ctx.count(8, [0, 1]) == 0


def test_count_batch_matches_individual_counts(ctx, oracle):
    inst = [(8, []), (9, [1]), (10, [2, 5]), (6, [0, 0]), (11, [3, 0, 7])]
    got = ctx.count_batch(inst)
    want = [oracle.known_count(8)] + [oracle.contract(n, symmetry=False, prefix=p)["count"] for n, p in inst[1:]]
    assert got == want


@pytest.mark.parametrize("merge", [1, 2])
def test_small_device_budget_splits_batches_and_stays_exact(ctx, oracle, merge):
    # Forced capacity pressure: batches split (and slices deepen) on the host.
    full = ctx.contract_rows(12, merge=merge)
    tight = ctx.contract_rows(12, merge=merge, device_budget_bytes=1536 << 10)
    assert full.device["batches"] == 1
    assert tight.device["batches"] > 1
    assert tight.count == full.count == oracle.known_count(12)


def test_deeper_host_slices_are_exact(ctx, oracle):
    for depth in [2, 3]:
        g = ctx.contract_rows(13, slice_depth=depth)
        assert g.count == oracle.known_count(13)
        assert g.device["slice_depth"] == depth
        # Merged rows after the host-seeded prefix equal the reference's frontier.
        o = oracle.contract(13)
        assert _gpu_layers(g) == _oracle_layers(o)


@pytest.mark.parametrize("n", [15, 17])
def test_full_size_counts(ctx, oracle, n):
    g = ctx.contract_rows(n)
    assert g.count == oracle.known_count(n)


@pytest.mark.parametrize("merge", [1, 2])
@pytest.mark.parametrize("n", [5, 8, 11, 12, 13])
def test_both_merge_strategies_match_oracle(ctx, oracle, qp, n, merge):
    g = ctx.contract_rows(n, merge=merge)
    assert g.device["merge"] == merge
    o = oracle.contract(n)
    assert g.count == o["count"]
    assert g.peak_states == o["peak_states"]
    assert _gpu_layers(g) == _oracle_layers(o)


def test_partition_merge_is_default_for_row_grain(ctx, qp):
    assert ctx.contract_rows(12).device["merge"] == qp.MERGE_PARTITION
    assert ctx.contract_rows(12, key_bits=128).device["merge"] == qp.MERGE_PARTITION
    assert ctx.contract_rows(9, granularity=1).device["merge"] == qp.MERGE_HASH
    with pytest.raises(qp.ContractionError):
        ctx.contract_rows(9, granularity=1, merge=qp.MERGE_PARTITION)


def test_n16_hash_and_partition_agree(ctx, golden):
    a = ctx.contract_rows(16, merge=1)
    b = ctx.contract_rows(16, merge=2)
    assert a.count == b.count == 14772512
    assert [(l.output_states, l.output_weight) for l in a.layers] == [(l.output_states, l.output_weight) for l in b.layers]
    assert b.peak_states == golden["e36_orbit_n16"]["16"]["peak_support"]


@pytest.mark.parametrize("n,k", [(6, 3), (8, 4), (10, 5), (12, 6), (13, 9), (14, 7)])
def test_slice_tail_is_exact(ctx, oracle, n, k):
    g = ctx.contract_rows(n, tail_row=k)
    assert g.device["tail_row"] == k
    assert g.count == oracle.known_count(n)
    o = oracle.contract(n)
    # Rows before the tail are the merged reference frontier.
    assert _gpu_layers(g)[:k] == _oracle_layers(o)[:k]


@pytest.mark.parametrize("n,k", [(10, 5), (12, 6), (13, 7), (14, 10)])
def test_slice_tail_row_statistics(ctx, oracle, n, k):
    # Row weights are linear in the boundary, so every tail row's output weight
    # equals the merged reference's; the first tail row reads exactly the
    # merged row-k boundary; later tail rows read at least the merged states
    # (independent batches merge less).
    g = ctx.contract_rows(n, tail_row=k)
    o = oracle.contract(n)
    assert [l.output_weight for l in g.layers] == [l["output_weight"] for l in o["layers"]]
    assert g.layers[k].input_states == o["layers"][k]["input_states"]
    assert g.layers[k].completed_row_terms == o["layers"][k]["completed_row_terms"]
    for row in range(k + 1, n):
        assert g.layers[row].input_states >= o["layers"][row]["input_states"]


@pytest.mark.parametrize("n,k", [(12, 2), (14, 2), (15, 3)])
def test_slice_tail_overflow_falls_back_to_row_engine(ctx, oracle, n, k):
    # Entries this early have frontiers far beyond one warp's shared memory:
    # they overflow and are contracted by the merged row engine instead.
    g = ctx.contract_rows(n, tail_row=k)
    assert g.device["tail_overflow"] > 0
    assert g.count == oracle.known_count(n)


def test_slice_tail_at_n17(ctx, oracle):
    g = ctx.contract_rows(17, tail_row=9)
    assert g.device["tail_row"] == 9 and g.device["tail_items"] > 0
    assert g.count == oracle.known_count(17)
    merged = ctx.contract_rows(17)
    assert merged.device["tail_row"] == 17 and merged.count == g.count


@pytest.mark.parametrize("key_bits", [64, 128])
@pytest.mark.parametrize("n", [9, 13])
def test_merge_counts_the_next_rows_terms(ctx, oracle, n, key_bits):
    """The partitioned merge counts the successor terms of the boundary it
    writes, so after the first device row an eager contraction runs no
    counting kernel: one count, then a scatter and a merge per row and batch,
    with every row's terms still equal to the oracle's."""
    g = ctx.contract_rows(n, key_bits=key_bits, use_graph=0)
    o = oracle.contract(n, backend=O.SORT_REDUCE)
    assert g.count == o["count"]
    assert _gpu_layers(g) == _oracle_layers(o)
    d = g.device
    device_rows = n - d["slice_depth"]
    assert d["gpu_launches"] == d["batches"] * (1 + 2 * device_rows)


@pytest.mark.parametrize("k,seed", [(6, 5), (7, 1022), (8, 9)])
def test_n22_compact_u64_keys_equal_u128_keys(ctx, qp, oracle, k, seed):
    """At N = 22 the u64 key drops the two always-clear diagonal bits (dr bit
    0, dl bit 21): every row of a prefix contraction equals the 128-bit-key
    run's and the global table's, the weights travel as exact 64-bit words,
    and a CUDA-graph replay repeats it."""
    prefix = _legal_prefix(22, k, seed)
    c64, r64 = ctx.count_with_stats(22, prefix, use_graph=0)
    c128, r128 = ctx.count_with_stats(22, prefix, key_bits=128)
    ctab, rtab = ctx.count_with_stats(22, prefix, merge=qp.MERGE_HASH)
    assert r64.device["key_bits"] == 64 and r64.device["exact_weights"]
    assert r128.device["key_bits"] == 128 and rtab.device["key_bits"] == 64
    assert c64 == c128 == ctab
    assert r64.peak_states == r128.peak_states == rtab.peak_states
    assert r64.device["entries_out"] == r128.device["entries_out"] == rtab.device["entries_out"]
    g1, _ = ctx.count_with_stats(22, prefix, use_graph=1)
    g2, rg = ctx.count_with_stats(22, prefix, use_graph=1)
    assert g1 == g2 == c64
    if k >= 7:
        want = oracle.contract(22, backend=oracle.PARALLEL_SORT_REDUCE, threads=8, symmetry=False, prefix=prefix)
        assert c64 == want["count"] and r64.peak_states == want["peak_states"]
