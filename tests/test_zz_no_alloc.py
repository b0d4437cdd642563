"""The row step that allocates no device memory, against the allocating API.

For callers that cannot call cudaMalloc (their framework's allocator owns the
GPU, or a serving loop must not synchronise on an allocation), the library
offers qpeps_row_step_noalloc: the caller owns the boundary buffers and the
merge scratch comes from a fixed array inside the library. This test drives a
whole contraction through that entry point, twice in a row (the scratch keeps
the previous call's contents), and checks every row and the count against
qpeps_contract_rows bit-exactly (integer results: no tolerance). It also
checks that an oversized step is rejected. This file is collected last.
"""
from __future__ import annotations

import ctypes

import pytest

pytestmark = pytest.mark.gpu

PRIMES = [2147483647, 2147483629, 2147483587, 2147483579]


def _crt(res, primes):
    value, mod = 0, 1
    for r, p in zip(res, primes):
        step = ((r - value) * pow(mod, -1, p)) % p
        value += mod * step
        mod *= p
    return value


def _step(lib, torch, n, R, keys, res, count):
    cap = max(n * count, 1)
    keys_out = torch.empty(cap, dtype=torch.int64, device="cuda")
    res_out = torch.empty(R * cap, dtype=torch.int32, device="cuda")
    out = ctypes.c_uint64(0)
    wres = (ctypes.c_uint64 * 4)()
    fres = (ctypes.c_uint64 * 4)()
    err = ctypes.create_string_buffer(512)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.qpeps_row_step_noalloc(n, R, keys.data_ptr(), res.data_ptr(), count, keys_out.data_ptr(),
                                    res_out.data_ptr(), cap, stream, ctypes.byref(out), wres, fres, err, len(err))
    assert rc == 0, err.value.decode()
    m = out.value
    next_keys = keys_out[:m].clone()
    next_res = res_out.view(R, cap)[:, :m].contiguous()
    return next_keys, next_res, m, _crt(list(wres)[:R], PRIMES[:R]), _crt(list(fres)[:R], PRIMES[:R])


def _contract_noalloc(lib, torch, n, R, rows=None):
    keys = torch.zeros(1, dtype=torch.int64, device="cuda")  # empty board, packed key 0
    res = torch.ones(R, 1, dtype=torch.int32, device="cuda")
    count = 1
    layers = []
    final = 0
    for _ in range(n if rows is None else rows):
        keys, res, count, weight, final = _step(lib, torch, n, R, keys, res, count)
        layers.append((count, weight))
    return layers, final


def _orbit_seed(torch, n, R):
    """Row 0 of the first-row vertical-reflection orbit path (src/lib.rs:721-749):
    a queen in column c < n-1-c weighs 2, the centre column of odd n weighs 1."""
    mask = (1 << n) - 1
    keys, weights = [], []
    for c in range(n):
        if c > n - 1 - c:
            continue
        b = 1 << c
        keys.append(b | (((b << 1) & mask) << n) | ((b >> 1) << (2 * n)))
        weights.append(2 if c < n - 1 - c else 1)
    k = torch.tensor(keys, dtype=torch.int64, device="cuda")
    r = torch.tensor([[w % p for w in weights] for p in PRIMES[:R]], dtype=torch.int32, device="cuda")
    return k, r, len(keys)


@pytest.mark.parametrize("n", [8, 12])
def test_noalloc_row_steps_match_contract_rows_twice(qp, n):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = qp.library()
    ref = qp.Context(0)
    try:
        want = ref.contract_rows(n, symmetry=0, merge=qp.MERGE_PARTITION)
    finally:
        ref.close()
    R = want.device["residues"]
    want_layers = [(l.output_states, l.output_weight) for l in want.layers]
    for _ in range(2):
        layers, count = _contract_noalloc(lib, torch, n, R)
        assert layers == want_layers
        assert count == want.count == qp.known_count(n)


def test_noalloc_rejects_a_step_beyond_its_scratch(qp):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = qp.library()
    n, R, m = 18, 2, 300_000  # 300k empty boards -> 5.4 M successor terms
    keys = torch.zeros(m, dtype=torch.int64, device="cuda")
    res = torch.ones(R * m, dtype=torch.int32, device="cuda")
    cap = n * m
    keys_out = torch.empty(cap, dtype=torch.int64, device="cuda")
    res_out = torch.empty(R * cap, dtype=torch.int32, device="cuda")
    out = ctypes.c_uint64(0)
    err = ctypes.create_string_buffer(512)
    rc = lib.qpeps_row_step_noalloc(n, R, keys.data_ptr(), res.data_ptr(), m, keys_out.data_ptr(), res_out.data_ptr(),
                                    cap, None, ctypes.byref(out), None, None, err, len(err))
    assert rc == qp.QPEPS_ERR_CAPACITY
    assert "no-allocation scratch holds at most" in err.value.decode()
    small = ctypes.c_uint64(0)
    rc = lib.qpeps_row_step_noalloc(n, R, keys.data_ptr(), res.data_ptr(), 10, keys_out.data_ptr(),
                                    res_out.data_ptr(), 5, None, ctypes.byref(small), None, None, err, len(err))
    assert rc == qp.QPEPS_ERR_CAPACITY
    assert "output capacity" in err.value.decode()


@pytest.mark.parametrize("n,R", [(9, 1), (10, 2), (11, 3), (10, 4)])
def test_noalloc_every_residue_count(qp, n, R):
    """One, two (16-byte candidates) and three or four (32-byte candidates)
    residue planes: whole contractions against qpeps_contract_rows with the
    same forced residue count, and the count against known_count."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = qp.library()
    ref = qp.Context(0)
    try:
        want = ref.contract_rows(n, symmetry=0, merge=qp.MERGE_PARTITION, residues=R)
    finally:
        ref.close()
    want_layers = [(l.output_states, l.output_weight) for l in want.layers]
    for _ in range(2):
        layers, count = _contract_noalloc(lib, torch, n, R)
        assert layers == want_layers
        assert count == qp.known_count(n)


def test_noalloc_step_near_its_term_limit(qp):
    """Q(14) on the orbit path, rows 1..8: the step into row 8 has 2,137,639
    successor terms, 87 % of the 2.456 M the 48 MiB scratch holds with two
    residue planes. Every row equals qpeps_contract_rows(14) bit-exactly."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = qp.library()
    n, R = 14, 2
    ref = qp.Context(0)
    try:
        want = ref.contract_rows(n)
    finally:
        ref.close()
    assert want.device["batches"] == 1
    want_layers = [(l.output_states, l.output_weight) for l in want.layers]
    assert want.layers[8].row_operator_matched == 2_137_639
    for _ in range(2):
        keys, res, count = _orbit_seed(torch, n, R)
        assert count == want_layers[0][0]
        for row in range(1, 9):
            keys, res, count, weight, _ = _step(lib, torch, n, R, keys, res, count)
            assert (count, weight) == want_layers[row], row
