"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this module; the product library never does.
"""
from __future__ import annotations

import ctypes
import subprocess
import threading
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

SORT_REDUCE = 0  # contract_rows_sort_reduce_with_modes (src/lib.rs:5287)
PARALLEL_SORT_REDUCE = 1  # contract_rows_parallel_sort_reduce_with_modes (5469)
HASH_COMPILED = 2  # contract_rows_with_backend(Compiled) (5633)
HASH_SITEWISE = 3  # contract_rows_with_backend(Sitewise) (5633)


class OqU128(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_uint64), ("hi", ctypes.c_uint64)]

    @property
    def value(self) -> int:
        return (int(self.hi) << 64) | int(self.lo)


def _u128(v: int) -> OqU128:
    return OqU128(v & ((1 << 64) - 1), v >> 64)


class OqLayer(ctypes.Structure):
    _fields_ = [
        ("row", ctypes.c_uint32),
        ("input_states", ctypes.c_uint64),
        ("tensor_entries_examined", OqU128),
        ("tensor_entries_matched", OqU128),
        ("row_operator_candidates", OqU128),
        ("row_operator_matched", OqU128),
        ("completed_row_terms", OqU128),
        ("output_states", ctypes.c_uint64),
        ("output_weight", OqU128),
        ("elapsed_s", ctypes.c_double),
        ("peak_rss_bytes", ctypes.c_uint64),
    ]


class OqResult(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint32),
        ("count", OqU128),
        ("elapsed_s", ctypes.c_double),
        ("peak_states", ctypes.c_uint64),
        ("tensor_entries_examined", OqU128),
        ("tensor_entries_matched", OqU128),
        ("row_operator_candidates", OqU128),
        ("row_operator_matched", OqU128),
        ("peak_rss_bytes", ctypes.c_uint64),
        ("n_layers", ctypes.c_uint32),
    ]


class OracleError(RuntimeError):
    pass


_lib = None
_lock = threading.Lock()


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


class OqExplicit(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint32),
        ("order", ctypes.c_uint32),
        ("complete", ctypes.c_uint32),
        ("pad", ctypes.c_uint32),
        ("count", OqU128),
        ("elapsed_s", ctypes.c_double),
        ("peak_states", ctypes.c_uint64),
        ("peak_open_bonds", ctypes.c_uint64),
        ("tensor_entries_examined", OqU128),
        ("tensor_entries_accepted", OqU128),
        ("contracted_sites", ctypes.c_uint64),
    ]


ROW_MAJOR = 0  # ExplicitFrontierOrder::RowMajor (src/lib.rs:940-944)
TOP_LEFT_DIAMOND = 1  # ExplicitFrontierOrder::TopLeftDiamond


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            if not LIB.exists():
                build()
            L = ctypes.CDLL(str(LIB))
            P = ctypes.POINTER
            L.oracle_contract.restype = ctypes.c_int
            L.oracle_contract.argtypes = [
                ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                P(ctypes.c_uint32), ctypes.c_uint32, P(OqResult), P(OqLayer), ctypes.c_uint32, P(OqU128),
                P(OqU128), ctypes.c_uint64, P(ctypes.c_uint64), ctypes.c_char_p, ctypes.c_size_t,
            ]
            L.oracle_known_count.argtypes = [ctypes.c_uint32, P(OqU128)]
            L.oracle_contract_from.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P(OqU128), P(OqU128),
                                               ctypes.c_uint64, P(OqResult), P(OqLayer), ctypes.c_uint32,
                                               ctypes.c_char_p, ctypes.c_size_t]
            L.oracle_dfs_count.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P(OqU128), ctypes.c_char_p, ctypes.c_size_t]
            L.oracle_brute_force_count.argtypes = [ctypes.c_uint32, P(OqU128)]
            L.oracle_crt_plan.argtypes = [ctypes.c_uint32, P(ctypes.c_uint64), P(ctypes.c_uint32), P(OqU128),
                                          P(OqU128), ctypes.c_char_p, ctypes.c_size_t]
            L.oracle_reconstruct_crt.argtypes = [P(ctypes.c_uint64), P(ctypes.c_uint64), ctypes.c_uint32, P(OqU128),
                                                 ctypes.c_char_p, ctypes.c_size_t]
            L.oracle_c_entries.argtypes = [P(ctypes.c_uint32), P(OqU128), ctypes.c_uint32]
            L.oracle_b_entries.argtypes = [P(ctypes.c_uint32), P(OqU128), ctypes.c_uint32]
            L.oracle_c_matching.argtypes = [ctypes.c_uint32] * 4
            L.oracle_compile_check.argtypes = [P(ctypes.c_uint32), P(ctypes.c_uint64), ctypes.c_uint32,
                                               ctypes.c_char_p, ctypes.c_size_t]
            L.oracle_pack.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, P(OqU128)]
            L.oracle_pack.restype = None
            L.oracle_unpack.argtypes = [ctypes.c_uint32, OqU128, P(ctypes.c_uint64), P(ctypes.c_uint64),
                                        P(ctypes.c_uint64)]
            L.oracle_unpack.restype = None
            L.oracle_row_terms.argtypes = [ctypes.c_uint32, ctypes.c_int, OqU128, P(OqU128), P(OqU128), ctypes.c_uint32]
            L.oracle_orbit_weight.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
            L.oracle_explicit_frontier.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, P(OqExplicit),
                                                   ctypes.c_char_p, ctypes.c_size_t]
            _lib = L
        return _lib


def contract(n: int, backend: int = SORT_REDUCE, symmetry: bool = True, sparse: bool = False, threads: int = 1,
             rows: int = 0, prefix=(), want_boundary: bool = False) -> dict:
    """Run one oracle driver; returns a dict shaped like ContractionResult."""
    L = lib()
    res = OqResult()
    cap = max(n, 1) + 1
    layers = (OqLayer * cap)()
    err = ctypes.create_string_buffer(512)
    pre = (ctypes.c_uint32 * max(len(prefix), 1))(*prefix)
    blen = ctypes.c_uint64(0)
    rc = L.oracle_contract(n, backend, int(symmetry), int(sparse), threads, rows, pre, len(prefix), ctypes.byref(res),
                           layers, cap, None, None, 0, ctypes.byref(blen) if want_boundary else None, err, len(err))
    if rc:
        raise OracleError(err.value.decode())
    out = {
        "n": res.n,
        "count": res.count.value,
        "elapsed": res.elapsed_s,
        "peak_states": res.peak_states,
        "tensor_entries_examined": res.tensor_entries_examined.value,
        "tensor_entries_matched": res.tensor_entries_matched.value,
        "row_operator_candidates": res.row_operator_candidates.value,
        "row_operator_matched": res.row_operator_matched.value,
        "layers": [
            {
                "row": layers[i].row,
                "input_states": layers[i].input_states,
                "tensor_entries_examined": layers[i].tensor_entries_examined.value,
                "tensor_entries_matched": layers[i].tensor_entries_matched.value,
                "row_operator_candidates": layers[i].row_operator_candidates.value,
                "row_operator_matched": layers[i].row_operator_matched.value,
                "completed_row_terms": layers[i].completed_row_terms.value,
                "output_states": layers[i].output_states,
                "output_weight": layers[i].output_weight.value,
                "elapsed": layers[i].elapsed_s,
            }
            for i in range(res.n_layers)
        ],
    }
    if want_boundary:
        m = blen.value
        keys = (OqU128 * max(m, 1))()
        weights = (OqU128 * max(m, 1))()
        rc = L.oracle_contract(n, backend, int(symmetry), int(sparse), threads, rows, pre, len(prefix),
                               ctypes.byref(res), layers, cap, keys, weights, m, ctypes.byref(blen), err, len(err))
        if rc:
            raise OracleError(err.value.decode())
        out["boundary"] = [(keys[i].value, weights[i].value) for i in range(m)]
    return out


def contract_from(n: int, row0: int, boundary) -> dict:
    """Contract rows [row0, n) from a list of (packed key, weight) pairs."""
    L = lib()
    m = len(boundary)
    keys = (OqU128 * max(m, 1))(*[_u128(k) for k, _ in boundary])
    ws = (OqU128 * max(m, 1))(*[_u128(w) for _, w in boundary])
    res = OqResult()
    cap = n + 1
    layers = (OqLayer * cap)()
    err = ctypes.create_string_buffer(512)
    if L.oracle_contract_from(n, row0, keys, ws, m, ctypes.byref(res), layers, cap, err, len(err)):
        raise OracleError(err.value.decode())
    return {
        "count": res.count.value,
        "peak_states": res.peak_states,
        "layers": [{"input_states": layers[i].input_states, "output_states": layers[i].output_states,
                    "completed_row_terms": layers[i].completed_row_terms.value} for i in range(res.n_layers)],
    }


def known_count(n: int):
    out = OqU128()
    return None if lib().oracle_known_count(n, ctypes.byref(out)) else out.value


def dfs_count(n: int, threads: int = 1) -> int:
    out = OqU128()
    err = ctypes.create_string_buffer(256)
    if lib().oracle_dfs_count(n, threads, ctypes.byref(out), err, len(err)):
        raise OracleError(err.value.decode())
    return out.value


def brute_force_count(n: int) -> int:
    out = OqU128()
    lib().oracle_brute_force_count(n, ctypes.byref(out))
    return out.value


def crt_plan(n: int):
    primes = (ctypes.c_uint64 * 4)()
    ln = ctypes.c_uint32()
    f = OqU128()
    p = OqU128()
    err = ctypes.create_string_buffer(256)
    if lib().oracle_crt_plan(n, primes, ctypes.byref(ln), ctypes.byref(f), ctypes.byref(p), err, len(err)):
        raise OracleError(err.value.decode())
    return list(primes)[: ln.value], f.value, p.value


def reconstruct_crt(residues, primes) -> int:
    m = len(residues)
    r = (ctypes.c_uint64 * max(m, 1))(*residues)
    p = (ctypes.c_uint64 * max(len(primes), 1))(*primes)
    out = OqU128()
    err = ctypes.create_string_buffer(256)
    if lib().oracle_reconstruct_crt(r, p, m, ctypes.byref(out), err, len(err)):
        raise OracleError(err.value.decode())
    return out.value


def c_entries():
    legs = (ctypes.c_uint32 * 32)()
    vals = (OqU128 * 32)()
    k = lib().oracle_c_entries(legs, vals, 32)
    return [(legs[i], vals[i].value) for i in range(k)]


def b_entries():
    raw = (ctypes.c_uint32 * 32)()
    vals = (OqU128 * 32)()
    k = lib().oracle_b_entries(raw, vals, 32)
    return [((raw[i] >> 8) & 1, raw[i] & 0xFF, vals[i].value) for i in range(k)]


def c_matching(column_in: int, row_in: int, dr_in: int, dl_in: int) -> int:
    return lib().oracle_c_matching(column_in, row_in, dr_in, dl_in)


def compile_check(entries) -> str | None:
    m = len(entries)
    legs = (ctypes.c_uint32 * max(m, 1))(*[e[0] for e in entries])
    vals = (ctypes.c_uint64 * max(m, 1))(*[e[1] for e in entries])
    err = ctypes.create_string_buffer(256)
    rc = lib().oracle_compile_check(legs, vals, m, err, len(err))
    return err.value.decode() if rc else None


def pack(n: int, cols: int, dr: int, dl: int) -> int:
    out = OqU128()
    lib().oracle_pack(n, cols, dr, dl, ctypes.byref(out))
    return out.value


def unpack(n: int, key: int):
    c, d, l = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    lib().oracle_unpack(n, _u128(key), ctypes.byref(c), ctypes.byref(d), ctypes.byref(l))
    return c.value, d.value, l.value


def row_terms(n: int, parent_key: int, sitewise: bool):
    keys = (OqU128 * 64)()
    w = (OqU128 * 64)()
    k = lib().oracle_row_terms(n, int(sitewise), _u128(parent_key), keys, w, 64)
    return [(keys[i].value, w[i].value) for i in range(k)]


def orbit_weight(n: int, column: int) -> int:
    return lib().oracle_orbit_weight(n, column)


def explicit_frontier(n: int, order: int = ROW_MAJOR, support_limit: int = 5_000_000) -> dict:
    """contract_explicit_c_frontier (src/lib.rs:961-967) restated; returns a
    dict shaped like ExplicitFrontierResult (count None when incomplete)."""
    out = OqExplicit()
    err = ctypes.create_string_buffer(512)
    if lib().oracle_explicit_frontier(n, order, support_limit, ctypes.byref(out), err, len(err)):
        raise OracleError(err.value.decode())
    return {
        "n": out.n,
        "order": out.order,
        "complete": bool(out.complete),
        "count": out.count.value if out.complete else None,
        "elapsed": out.elapsed_s,
        "peak_states": out.peak_states,
        "peak_open_bonds": out.peak_open_bonds,
        "tensor_entries_examined": out.tensor_entries_examined.value,
        "tensor_entries_accepted": out.tensor_entries_accepted.value,
        "contracted_sites": out.contracted_sites,
    }
