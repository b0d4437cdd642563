"""Serving: continuous batching of counting requests of mixed N and prefixes.

Every result of a mixed stream is checked bit-exactly against the CPU oracle
(the reference's contraction from the placed prefix) and against the same
request run alone through qpeps_count, i.e. the same alone and in the mix.
"""
from __future__ import annotations

import random
import time

import pytest

pytestmark = pytest.mark.gpu


def _oracle_count(oracle, n, prefix):
    return oracle.known_count(n) if not prefix else oracle.contract(n, symmetry=False, prefix=prefix)["count"]


def test_mixed_stream_is_exact_and_batched(qp, ctx, oracle):
    rng = random.Random(20261203)
    reqs = []
    for tag in range(240):
        n = rng.randint(5, 13)
        k = rng.randint(0, 3)
        reqs.append((tag, n, qp.random_prefix(rng, n, k)))
    got = {}
    with qp.Server(0, use_cache=0, max_slots=32) as sv:
        for tag, n, prefix in reqs:
            sv.submit(n, prefix, tag)
            if tag % 17 == 0:
                time.sleep(0.002)  # arrivals spread while earlier requests run
            for c in sv.poll():
                got[c["tag"]] = c
        deadline = time.time() + 120
        while len(got) < len(reqs) and time.time() < deadline:
            for c in sv.poll(wait_ms=100):
                got[c["tag"]] = c
        stats = sv.stats()
    assert len(got) == len(reqs)
    for tag, n, prefix in reqs:
        c = got[tag]
        assert c["status"] == 0
        assert c["count"] == _oracle_count(oracle, n, prefix), (n, prefix)
        assert c["count"] == ctx.count(n, prefix), (n, prefix)
    # Requests shared steps: far fewer batch steps than rows contracted.
    total_rows = sum(n - len(p) for _, n, p in reqs)
    assert stats["batch_steps"] < total_rows / 4
    assert stats["completed"] == len(reqs)


def test_large_requests_run_beside_the_batch(qp, oracle):
    rng = random.Random(7)
    with qp.Server(0, use_cache=0, large_threshold_states=50_000) as sv:
        sv.submit(14, [], 1)          # estimated frontier above the threshold: large path
        sv.submit(13, [2], 2)         # large path too (estimate ~80k)
        for tag in range(3, 40):
            n = rng.randint(6, 11)
            sv.submit(n, qp.random_prefix(rng, n, rng.randint(0, 3)), tag)
        got = {}
        deadline = time.time() + 120
        while len(got) < 39 and time.time() < deadline:
            for c in sv.poll(wait_ms=100):
                got[c["tag"]] = c
    assert got[1]["path"] == "large" and got[1]["count"] == oracle.known_count(14)
    assert got[2]["count"] == oracle.contract(13, symmetry=False, prefix=[2])["count"]
    assert any(c["path"] == "batch" for c in got.values())


def test_cache_answers_repeats_and_mirrors(qp, oracle):
    with qp.Server(0, use_cache=1) as sv:
        sv.submit(10, [1, 4], 1)
        first = None
        deadline = time.time() + 60
        while first is None and time.time() < deadline:
            for c in sv.poll(wait_ms=100):
                first = c
        sv.submit(10, [8, 5], 2)  # mirror image of [1, 4]
        second = None
        while second is None and time.time() < deadline:
            for c in sv.poll(wait_ms=100):
                second = c
    want = oracle.contract(10, symmetry=False, prefix=[1, 4])["count"]
    assert first["count"] == second["count"] == want
    assert second["path"] == "cache"


def test_trivial_prefixes(qp):
    with qp.Server(0, use_cache=0) as sv:
        sv.submit(8, [0, 4, 7, 5, 2, 6, 1, 3], 1)  # a complete solution
        sv.submit(8, [0, 1], 2)                    # attacked
        got = {}
        deadline = time.time() + 30
        while len(got) < 2 and time.time() < deadline:
            for c in sv.poll(wait_ms=100):
                got[c["tag"]] = c
    assert got[1]["count"] == 1 and got[2]["count"] == 0


def test_batch_over_budget_moves_requests_to_large_context(qp, oracle):
    # A 1 MiB shared batch cannot hold these requests' frontiers: the batch
    # gives them to the large-request context, which finishes them exactly.
    rng = random.Random(11)
    reqs = [(tag, 13, qp.random_prefix(rng, 13, 1)) for tag in range(12)]
    got = {}
    with qp.Server(0, use_cache=0, batch_budget_bytes=1 << 20, large_threshold_states=10**12) as sv:
        for tag, n, prefix in reqs:
            sv.submit(n, prefix, tag)
        deadline = time.time() + 120
        while len(got) < len(reqs) and time.time() < deadline:
            for c in sv.poll(wait_ms=100):
                got[c["tag"]] = c
        stats = sv.stats()
    assert len(got) == len(reqs)
    assert stats["batch_requeued"] > 0
    for tag, n, prefix in reqs:
        assert got[tag]["status"] == 0
        assert got[tag]["count"] == _oracle_count(oracle, n, prefix), (n, prefix)


def test_identical_requests_in_flight_are_coalesced(qp):
    with qp.Server(0, use_cache=1) as sv:
        for tag in range(6):
            sv.submit(15, [], tag)          # identical
        sv.submit(15, [3], 10)
        sv.submit(15, [11], 11)             # mirror of [3]
        got = {}
        deadline = time.time() + 120
        while len(got) < 8 and time.time() < deadline:
            for c in sv.poll(wait_ms=100):
                got[c["tag"]] = c
        stats = sv.stats()
    assert len(got) == 8
    assert all(got[t]["count"] == qp.known_count(15) for t in range(6))
    assert got[10]["count"] == got[11]["count"]
    assert stats["coalesced"] + stats["cache_hits"] == 6
    assert stats["coalesced"] >= 1
    assert {got[t]["path"] for t in range(6)} - {"batch", "large", "cache", "coalesced"} == set()


@pytest.mark.parametrize("workers", [1, 3])
def test_several_large_workers_answer_exactly(qp, oracle, workers):
    # Large requests run on `workers` contexts at once; every answer equals
    # the same request contracted alone, whichever worker ran it.
    reqs = [(14, []), (13, [2]), (14, [5]), (13, []), (14, [1, 8]), (12, [])]
    with qp.Server(0, use_cache=0, large_threshold_states=20_000, large_workers=workers) as sv:
        for tag, (n, prefix) in enumerate(reqs):
            sv.submit(n, prefix, tag)
        got = {}
        for _ in range(600):
            for c in sv.poll(wait_ms=50):
                got[c["tag"]] = c
            if len(got) == len(reqs):
                break
        stats = sv.stats()
    assert len(got) == len(reqs)
    assert stats["large_runs"] >= 4
    ctx = qp.Context(0)
    try:
        for tag, (n, prefix) in enumerate(reqs):
            assert got[tag]["status"] == 0
            assert got[tag]["count"] == ctx.count(n, prefix)
    finally:
        ctx.close()
