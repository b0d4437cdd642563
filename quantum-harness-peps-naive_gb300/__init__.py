"""GB300 exact N-Queens PEPS row-boundary contraction: Python mirror of the
reference library API over the C ABI in include/qpeps.h.

Reference (Rust crate ``nqueens-peps-naive``):

* ``contract_rows(n) -> Result<ContractionResult, String>``  src/lib.rs:758
* ``known_count(n) -> Option<u128>``                          src/lib.rs:5752-5784
* ``ContractionResult`` / ``LayerMetric``                     src/lib.rs:388-415

``contract_rows`` returns the same fields with the same meaning and raises
``ContractionError`` where the reference returns ``Err(String)`` (same
message text, e.g. N > 42). The device library must be built
(``buildlib.py``); there is no CPU fallback: importing the module on a machine
without the library or without a CUDA device raises when a context is
needed.
"""
from __future__ import annotations

import ctypes
import dataclasses
import threading
from pathlib import Path
from typing import Iterable, Sequence

_PKG = Path(__file__).resolve().parent
LIBRARY_PATH = _PKG / "libqpeps.so"

QPEPS_OK = 0
QPEPS_ERR_RANGE = 1
QPEPS_ERR_OOM = 2
QPEPS_ERR_CAPACITY = 3
QPEPS_ERR_CRT_BOUND = 4
QPEPS_ERR_CUDA = 5
QPEPS_ERR_INVALID = 6
QPEPS_ERR_OVERFLOW = 7
QPEPS_ERR_TIMEOUT = 8

GRAIN_ROW = 0
GRAIN_SITE = 1
MERGE_AUTO = 0
MERGE_HASH = 1
MERGE_PARTITION = 2
SCATTER_SEARCH = 0
SCATTER_WINDOW = 1
SCATTER_TWO_LEVEL = 2
SCATTER_CLASS = 3
SCATTER_DIRECT = 4
MERGEK_SCAN = 0
MERGEK_CLAIM = 1


class U128(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_uint64), ("hi", ctypes.c_uint64)]

    @property
    def value(self) -> int:
        return (int(self.hi) << 64) | int(self.lo)


class Layer(ctypes.Structure):
    _fields_ = [
        ("row", ctypes.c_uint32),
        ("input_states", ctypes.c_uint64),
        ("tensor_entries_examined", U128),
        ("tensor_entries_matched", U128),
        ("row_operator_candidates", U128),
        ("row_operator_matched", U128),
        ("completed_row_terms", U128),
        ("output_states", ctypes.c_uint64),
        ("output_weight", U128),
        ("elapsed_s", ctypes.c_double),
        ("peak_rss_bytes", ctypes.c_uint64),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint32),
        ("count", U128),
        ("elapsed_s", ctypes.c_double),
        ("peak_states", ctypes.c_uint64),
        ("tensor_entries_examined", U128),
        ("tensor_entries_matched", U128),
        ("row_operator_candidates", U128),
        ("row_operator_matched", U128),
        ("peak_rss_bytes", ctypes.c_uint64),
        ("n_layers", ctypes.c_uint32),
        ("residues", ctypes.c_uint32),
        ("key_bits", ctypes.c_uint32),
        ("slice_depth", ctypes.c_uint32),
        ("batches", ctypes.c_uint32),
        ("merge", ctypes.c_uint32),
        ("entries_in", ctypes.c_uint64),
        ("entries_out", ctypes.c_uint64),
        ("candidates", ctypes.c_uint64),
        ("gpu_launches", ctypes.c_uint64),
        ("peak_device_bytes", ctypes.c_uint64),
        ("device_ms", ctypes.c_double),
        ("merge_kernel_ms", ctypes.c_double),
        ("scatter_kernel_ms", ctypes.c_double),
        ("merge_kernel_launches", ctypes.c_uint64),
        ("merge_kernel_bytes", ctypes.c_uint64),
        ("tail_row", ctypes.c_uint32),
        ("exact_weights", ctypes.c_uint32),
        ("tail_items", ctypes.c_uint64),
        ("tail_overflow", ctypes.c_uint64),
        ("tail_kernel_ms", ctypes.c_double),
        ("h2d_bytes", ctypes.c_uint64),
        ("d2h_bytes", ctypes.c_uint64),
        ("residue_primes", ctypes.c_uint32 * 4),
        ("count_residues", ctypes.c_uint64 * 4),
    ]


class Options(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("granularity", ctypes.c_uint32),
        ("merge", ctypes.c_uint32),
        ("residues", ctypes.c_uint32),
        ("key_bits", ctypes.c_uint32),
        ("slice_depth", ctypes.c_uint32),
        ("symmetry", ctypes.c_uint32),
        ("collect_layers", ctypes.c_uint32),
        ("block_threads", ctypes.c_uint32),
        ("use_graph", ctypes.c_uint32),
        ("device_budget_bytes", ctypes.c_uint64),
        ("tail_row", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]


class ServeConfig(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("max_slots", ctypes.c_uint32),
        ("batch_budget_bytes", ctypes.c_uint64),
        ("large_budget_bytes", ctypes.c_uint64),
        ("large_threshold_states", ctypes.c_uint64),
        ("use_cache", ctypes.c_uint32),
        ("large_workers", ctypes.c_uint32),
    ]


class ServeCompletion(ctypes.Structure):
    _fields_ = [
        ("tag", ctypes.c_uint64),
        ("count", U128),
        ("status", ctypes.c_int32),
        ("n", ctypes.c_uint32),
        ("k", ctypes.c_uint32),
        ("path", ctypes.c_uint32),
        ("latency_s", ctypes.c_double),
        ("queue_s", ctypes.c_double),
    ]


class ServeStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64)
                for f in ("submitted", "completed", "batch_steps", "cache_hits", "large_runs", "batch_requeued",
                          "coalesced")]


PROBE_APPEND = 0
PROBE_STORE = 1
PROBE_ATOMIC = 2
PROBE_STREAM = 3
PROBE_APPEND_PLAIN = 4
ORDER_ROW_MAJOR = 0
ORDER_TOP_LEFT_DIAMOND = 1


class ExplicitResult(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint32),
        ("order", ctypes.c_uint32),
        ("complete", ctypes.c_uint32),
        ("merge", ctypes.c_uint32),
        ("count", U128),
        ("elapsed_s", ctypes.c_double),
        ("peak_states", ctypes.c_uint64),
        ("peak_open_bonds", ctypes.c_uint64),
        ("tensor_entries_examined", U128),
        ("tensor_entries_accepted", U128),
        ("contracted_sites", ctypes.c_uint64),
        ("peak_rss_bytes", ctypes.c_uint64),
        ("gpu_launches", ctypes.c_uint64),
        ("device_ms", ctypes.c_double),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("scatter_kind", ctypes.c_uint32),
        ("parents_per_lane", ctypes.c_uint32),
        ("merge_kind", ctypes.c_uint32),
        ("wide_merge", ctypes.c_uint32),
        ("wide_above_parts", ctypes.c_uint32),
        ("spread_cursors_below", ctypes.c_uint32),
        ("fold_weights", ctypes.c_uint32),
        ("partition_fill", ctypes.c_double),
        ("slice_margin", ctypes.c_double),
        ("unit_target", ctypes.c_uint32),
        ("unit_sample", ctypes.c_uint32),
        ("batch_lanes", ctypes.c_uint32),
        ("merge_compact", ctypes.c_uint32),
        ("scatter_block", ctypes.c_uint32),
        ("merge_auto", ctypes.c_uint32),
        ("slice_rows", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f not in ("struct_size", "reserved")}


# Every symbol include/qpeps.h declares, with its ctypes signature.
_VP = ctypes.c_void_p
_SIGNATURES = {
    "qpeps_version": (ctypes.c_char_p, []),
    "qpeps_options_default": (None, [ctypes.POINTER(Options)]),
    "qpeps_known_count": (ctypes.c_int, [ctypes.c_uint32, ctypes.POINTER(U128)]),
    "qpeps_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_VP), ctypes.c_char_p, ctypes.c_size_t]),
    "qpeps_ctx_destroy": (None, [_VP]),
    "qpeps_contract_rows": (
        ctypes.c_int,
        [_VP, ctypes.c_uint32, ctypes.POINTER(Options), ctypes.POINTER(Result), ctypes.POINTER(Layer),
         ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "qpeps_count": (
        ctypes.c_int,
        [_VP, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32, ctypes.POINTER(Options),
         ctypes.POINTER(U128), ctypes.POINTER(Result), ctypes.c_char_p, ctypes.c_size_t],
    ),
    "qpeps_count_batch": (
        ctypes.c_int,
        [_VP, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
         ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(Options),
         ctypes.POINTER(U128), ctypes.c_char_p, ctypes.c_size_t],
    ),
    "qpeps_row_step_noalloc": (
        ctypes.c_int,
        [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
         ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64), ctypes.c_char_p, ctypes.c_size_t],
    ),
    "qpeps_serve_config_default": (None, [ctypes.POINTER(ServeConfig)]),
    "qpeps_serve_open": (
        ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ServeConfig), ctypes.POINTER(_VP), ctypes.c_char_p, ctypes.c_size_t]
    ),
    "qpeps_serve_submit": (
        ctypes.c_int,
        [_VP, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32, ctypes.c_uint64, ctypes.c_char_p,
         ctypes.c_size_t],
    ),
    "qpeps_serve_poll": (
        ctypes.c_int,
        [_VP, ctypes.POINTER(ServeCompletion), ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32],
    ),
    "qpeps_serve_stats_get": (ctypes.c_int, [_VP, ctypes.POINTER(ServeStats)]),
    "qpeps_serve_error": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_size_t]),
    "qpeps_serve_close": (None, [_VP]),
    "qpeps_explicit_frontier": (
        ctypes.c_int,
        [_VP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(ExplicitResult), ctypes.c_char_p,
         ctypes.c_size_t],
    ),
    "qpeps_tuning_default": (None, [ctypes.POINTER(Tuning)]),
    "qpeps_ctx_get_tuning": (ctypes.c_int, [_VP, ctypes.POINTER(Tuning)]),
    "qpeps_ctx_set_tuning": (ctypes.c_int, [_VP, ctypes.POINTER(Tuning), ctypes.c_char_p, ctypes.c_size_t]),
    "qpeps_autotune": (
        ctypes.c_int,
        [_VP, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(Tuning), ctypes.POINTER(ctypes.c_double),
         ctypes.c_char_p, ctypes.c_size_t],
    ),
    "qpeps_ctx_device_name": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_size_t]),
    "qpeps_probe_append": (
        ctypes.c_int,
        [_VP, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double),
         ctypes.c_char_p, ctypes.c_size_t],
    ),
    "qpeps_certify_c": (
        ctypes.c_int,
        [ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32, ctypes.c_char_p,
         ctypes.c_size_t],
    ),
}

_lib = None
_lib_lock = threading.Lock()


def library() -> ctypes.CDLL:
    """Load libqpeps.so (raises if it has not been built)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not LIBRARY_PATH.exists():
                raise ContractionError(QPEPS_ERR_CUDA, f"device library not built: {LIBRARY_PATH}")
            lib = ctypes.CDLL(str(LIBRARY_PATH))
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
        return _lib


class ContractionError(RuntimeError):
    """The reference's ``Err(String)``; ``code`` is the QPEPS_ERR_* value."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code
        self.message = message


def _check(rc: int, err: ctypes.Array) -> None:
    if rc != QPEPS_OK:
        raise ContractionError(rc, err.value.decode(errors="replace"))


@dataclasses.dataclass
class LayerMetric:
    """src/lib.rs:388-401 (``row`` is 0-based)."""

    row: int
    input_states: int
    tensor_entries_examined: int
    tensor_entries_matched: int
    row_operator_candidates: int
    row_operator_matched: int
    completed_row_terms: int
    output_states: int
    output_weight: int
    elapsed: float
    peak_rss_bytes: int


@dataclasses.dataclass
class ContractionResult:
    """src/lib.rs:403-415 plus device-side facts in ``device``."""

    n: int
    count: int
    elapsed: float
    peak_states: int
    tensor_entries_examined: int
    tensor_entries_matched: int
    row_operator_candidates: int
    row_operator_matched: int
    peak_rss_bytes: int
    layers: list
    device: dict


def options(**kw) -> Options:
    """Options with the library defaults, overridden by keyword."""
    o = Options()
    library().qpeps_options_default(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k) or k == "struct_size":
            raise TypeError(f"unknown option {k}")
        setattr(o, k, int(v))
    return o


def _result_from(res: Result, layers: Sequence[Layer] | None) -> ContractionResult:
    lay = []
    if layers is not None:
        for i in range(min(res.n_layers, len(layers))):
            L = layers[i]
            lay.append(
                LayerMetric(
                    row=L.row,
                    input_states=L.input_states,
                    tensor_entries_examined=L.tensor_entries_examined.value,
                    tensor_entries_matched=L.tensor_entries_matched.value,
                    row_operator_candidates=L.row_operator_candidates.value,
                    row_operator_matched=L.row_operator_matched.value,
                    completed_row_terms=L.completed_row_terms.value,
                    output_states=L.output_states,
                    output_weight=L.output_weight.value,
                    elapsed=L.elapsed_s,
                    peak_rss_bytes=L.peak_rss_bytes,
                )
            )
    device = {
        "residues": res.residues,
        "key_bits": res.key_bits,
        "slice_depth": res.slice_depth,
        "batches": res.batches,
        "merge": res.merge,
        "entries_in": res.entries_in,
        "entries_out": res.entries_out,
        "candidates": res.candidates,
        "gpu_launches": res.gpu_launches,
        "peak_device_bytes": res.peak_device_bytes,
        "device_ms": res.device_ms,
        "merge_kernel_ms": res.merge_kernel_ms,
        "scatter_kernel_ms": res.scatter_kernel_ms,
        "merge_kernel_launches": res.merge_kernel_launches,
        "merge_kernel_bytes": res.merge_kernel_bytes,
        "tail_row": res.tail_row,
        "exact_weights": res.exact_weights,
        "tail_items": res.tail_items,
        "tail_overflow": res.tail_overflow,
        "tail_kernel_ms": res.tail_kernel_ms,
        "h2d_bytes": res.h2d_bytes,
        "d2h_bytes": res.d2h_bytes,
        "residue_primes": list(res.residue_primes)[: res.residues],
        "count_residues": list(res.count_residues)[: res.residues],
    }
    return ContractionResult(
        n=res.n,
        count=res.count.value,
        elapsed=res.elapsed_s,
        peak_states=res.peak_states,
        tensor_entries_examined=res.tensor_entries_examined.value,
        tensor_entries_matched=res.tensor_entries_matched.value,
        row_operator_candidates=res.row_operator_candidates.value,
        row_operator_matched=res.row_operator_matched.value,
        peak_rss_bytes=res.peak_rss_bytes,
        layers=lay,
        device=device,
    )


class Context:
    """One CUDA device and its device-memory pool (``qpeps_ctx``)."""

    def __init__(self, device: int = 0):
        lib = library()
        err = ctypes.create_string_buffer(4096)
        h = _VP()
        _check(lib.qpeps_ctx_create(device, ctypes.byref(h), err, len(err)), err)
        self._h = h
        self._lock = threading.Lock()

    def close(self) -> None:
        if getattr(self, "_h", None):
            library().qpeps_ctx_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def contract_rows(self, n: int, **opts) -> ContractionResult:
        """Replaces ``contract_rows(n)`` (src/lib.rs:758)."""
        lib = library()
        o = options(**opts)
        res = Result()
        cap = max(int(n), 1)
        layers = (Layer * cap)()
        err = ctypes.create_string_buffer(4096)
        with self._lock:
            rc = lib.qpeps_contract_rows(self._h, int(n), ctypes.byref(o), ctypes.byref(res), layers, cap, err, len(err))
        _check(rc, err)
        return _result_from(res, layers)

    def count(self, n: int, prefix: Sequence[int] = (), **opts) -> int:
        """Completions of a board with ``len(prefix)`` rows placed."""
        c, _ = self.count_with_stats(n, prefix, **opts)
        return c

    def count_with_stats(self, n: int, prefix: Sequence[int] = (), **opts):
        lib = library()
        o = options(**opts)
        k = len(prefix)
        arr = (ctypes.c_uint32 * max(k, 1))(*prefix)
        out = U128()
        res = Result()
        err = ctypes.create_string_buffer(4096)
        with self._lock:
            rc = lib.qpeps_count(self._h, int(n), arr if k else None, k, ctypes.byref(o), ctypes.byref(out),
                                 ctypes.byref(res), err, len(err))
        _check(rc, err)
        return out.value, _result_from(res, None)

    def count_batch(self, instances: Iterable[tuple[int, Sequence[int]]], **opts) -> list[int]:
        lib = library()
        inst = list(instances)
        num = len(inst)
        ns = (ctypes.c_uint32 * max(num, 1))(*[i[0] for i in inst])
        ks = (ctypes.c_uint32 * max(num, 1))(*[len(i[1]) for i in inst])
        offs = []
        cols = []
        for _, pre in inst:
            offs.append(len(cols))
            cols.extend(pre)
        po = (ctypes.c_uint32 * max(num, 1))(*offs)
        pc = (ctypes.c_uint32 * max(len(cols), 1))(*cols)
        counts = (U128 * max(num, 1))()
        o = options(**opts)
        err = ctypes.create_string_buffer(4096)
        with self._lock:
            rc = lib.qpeps_count_batch(self._h, num, ns, ks, po, pc, ctypes.byref(o), counts, err, len(err))
        _check(rc, err)
        return [counts[i].value for i in range(num)]


    def explicit_frontier(self, n: int, order: int = ORDER_ROW_MAJOR, support_limit: int = 5_000_000) -> dict:
        """Replaces ``contract_explicit_c_frontier(n, order, support_limit)``
        (src/lib.rs:961-967); ``count`` is None when the result is incomplete."""
        out = ExplicitResult()
        err = ctypes.create_string_buffer(4096)
        with self._lock:
            rc = library().qpeps_explicit_frontier(self._h, int(n), int(order), int(support_limit), ctypes.byref(out),
                                                   err, len(err))
        _check(rc, err)
        return {
            "n": out.n,
            "order": out.order,
            "complete": bool(out.complete),
            "merge": out.merge,
            "count": out.count.value if out.complete else None,
            "elapsed": out.elapsed_s,
            "peak_states": out.peak_states,
            "peak_open_bonds": out.peak_open_bonds,
            "tensor_entries_examined": out.tensor_entries_examined.value,
            "tensor_entries_accepted": out.tensor_entries_accepted.value,
            "contracted_sites": out.contracted_sites,
            "peak_rss_bytes": out.peak_rss_bytes,
            "gpu_launches": out.gpu_launches,
            "device_ms": out.device_ms,
        }

    # ---- tuning (no reference counterpart) ---------------------------------
    @property
    def tuning(self) -> dict:
        t = Tuning()
        rc = library().qpeps_ctx_get_tuning(self._h, ctypes.byref(t))
        if rc != QPEPS_OK:
            raise ContractionError(rc, "qpeps_ctx_get_tuning failed")
        return t.as_dict()

    def set_tuning(self, **kw) -> dict:
        """Change tuning fields (see ``qpeps_tuning``); returns the new tuning."""
        t = Tuning()
        library().qpeps_ctx_get_tuning(self._h, ctypes.byref(t))
        for k, v in kw.items():
            if k not in t.as_dict():
                raise ContractionError(QPEPS_ERR_INVALID, f"unknown tuning field {k}")
            setattr(t, k, v)
        err = ctypes.create_string_buffer(4096)
        with self._lock:
            rc = library().qpeps_ctx_set_tuning(self._h, ctypes.byref(t), err, len(err))
        _check(rc, err)
        return self.tuning

    @property
    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        library().qpeps_ctx_device_name(self._h, buf, len(buf))
        return buf.value.decode(errors="replace")

    def tuning_key(self, n: int) -> str:
        """Autotuner cache key: device name, library version and probe size."""
        return f"{self.device_name}|{version()}|n={int(n)}"

    def load_tuning(self, n: int, cache: str | Path) -> dict | None:
        """Apply the cached autotuner result for this device and library
        version, probed at ``n`` or else at the largest smaller size (no
        search); returns the cache entry, or None when the cache holds none."""
        import json

        try:
            entries = json.loads(Path(cache).read_text())
        except (OSError, ValueError):
            return None
        # The entry of this N, else of the largest probe size below it.
        key = None
        for m in range(int(n), 7, -1):
            if self.tuning_key(m) in entries:
                key = self.tuning_key(m)
                break
        if key is None:
            return None
        e = entries[key]
        self.set_tuning(**e["tuning"])
        return {"key": key, **e}

    def autotune(self, n: int = 16, repeats: int = 2, cache: str | Path | None = None) -> dict:
        """Pick the fastest tuning for this device (``qpeps_autotune`` on a
        probe contraction of size ``n``). With ``cache``, a JSON file keyed
        by device name, library version and ``n`` is read first and updated
        after a search. Returns ``{"tuning": {...}, "device_ms": ms,
        "cached": bool}``."""
        import json

        key = self.tuning_key(n)
        path = Path(cache) if cache is not None else None
        entries = {}
        if path is not None and path.exists():
            try:
                entries = json.loads(path.read_text())
            except (OSError, ValueError):
                entries = {}
            if key in entries:
                self.set_tuning(**entries[key]["tuning"])
                return {"tuning": self.tuning, "device_ms": entries[key]["device_ms"], "cached": True}
        t = Tuning()
        ms = ctypes.c_double()
        err = ctypes.create_string_buffer(4096)
        with self._lock:
            rc = library().qpeps_autotune(self._h, int(n), int(repeats), ctypes.byref(t), ctypes.byref(ms), err,
                                          len(err))
        _check(rc, err)
        out = {"tuning": t.as_dict(), "device_ms": ms.value, "cached": False}
        if path is not None:
            entries[key] = {"tuning": out["tuning"], "device_ms": out["device_ms"]}
            path.write_text(json.dumps(entries, indent=1, sort_keys=True))
        return out

    def probe_append(self, mode: int, candidates: int, parts: int, repeats: int = 3) -> float:
        """Best device time (ms) of the scatter's memory pattern alone
        (``qpeps_probe_append``): ``candidates`` pseudo-random 16-byte records
        into ``parts`` partitions of 2048 slots by ``mode`` (PROBE_APPEND,
        PROBE_STORE, PROBE_ATOMIC, PROBE_STREAM or PROBE_APPEND_PLAIN)."""
        ms = ctypes.c_double()
        err = ctypes.create_string_buffer(4096)
        with self._lock:
            rc = library().qpeps_probe_append(self._h, int(mode), int(candidates), int(parts), int(repeats),
                                              ctypes.byref(ms), err, len(err))
        _check(rc, err)
        return ms.value


def tuning_default() -> dict:
    """The library's default tuning (``qpeps_tuning_default``)."""
    t = Tuning()
    library().qpeps_tuning_default(ctypes.byref(t))
    return t.as_dict()


class Server:
    """Continuous-batching counting server (qpeps_serve_*)."""

    PATHS = {0: "batch", 1: "large", 2: "cache", 3: "host", 4: "coalesced"}

    def __init__(self, device: int = 0, **cfg):
        lib = library()
        c = ServeConfig()
        lib.qpeps_serve_config_default(ctypes.byref(c))
        for k, v in cfg.items():
            if not hasattr(c, k) or k == "struct_size":
                raise TypeError(f"unknown serve option {k}")
            setattr(c, k, int(v))
        err = ctypes.create_string_buffer(4096)
        h = _VP()
        _check(lib.qpeps_serve_open(device, ctypes.byref(c), ctypes.byref(h), err, len(err)), err)
        self._h = h

    def submit(self, n: int, prefix: Sequence[int] = (), tag: int = 0) -> None:
        k = len(prefix)
        arr = (ctypes.c_uint32 * max(k, 1))(*prefix)
        err = ctypes.create_string_buffer(4096)
        _check(library().qpeps_serve_submit(self._h, n, arr if k else None, k, tag, err, len(err)), err)

    def poll(self, max_items: int = 1024, wait_ms: int = 0) -> list[dict]:
        buf = (ServeCompletion * max_items)()
        got = ctypes.c_uint32(0)
        rc = library().qpeps_serve_poll(self._h, buf, max_items, ctypes.byref(got), wait_ms)
        out = [
            {"tag": b.tag, "count": b.count.value, "status": b.status, "n": b.n, "k": b.k,
             "path": self.PATHS.get(b.path, b.path), "latency_s": b.latency_s, "queue_s": b.queue_s}
            for b in buf[: got.value]
        ]
        if rc != QPEPS_OK:
            err = ctypes.create_string_buffer(4096)
            code = library().qpeps_serve_error(self._h, err, len(err))
            raise ContractionError(code or rc, "server stopped: " + err.value.decode(errors="replace"))
        return out

    def stats(self) -> dict:
        st = ServeStats()
        library().qpeps_serve_stats_get(self._h, ctypes.byref(st))
        return {f: getattr(st, f) for f, _ in ServeStats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            library().qpeps_serve_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def random_prefix(rng, n: int, k: int) -> list[int]:
    """k queens placed row by row, each column drawn uniformly from the
    non-attacked columns of its row; the whole prefix is redrawn when a row has
    no legal column."""
    while True:
        cols, dr, dl, out = 0, 0, 0, []
        mask = (1 << n) - 1
        ok = True
        for _ in range(k):
            free = [c for c in range(n) if not ((cols | dr | dl) >> c) & 1]
            if not free:
                ok = False
                break
            c = rng.choice(free)
            b = 1 << c
            cols, dr, dl = cols | b, ((dr | b) << 1) & mask, (dl | b) >> 1
            out.append(c)
        if ok:
            return out


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def contract_rows(n: int, **opts) -> ContractionResult:
    """``contract_rows(n)`` (src/lib.rs:758) on the default device."""
    return default_context().contract_rows(n, **opts)


def count(n: int, prefix: Sequence[int] = (), **opts) -> int:
    return default_context().count(n, prefix, **opts)


def known_count(n: int) -> int | None:
    """``known_count`` (src/lib.rs:5752-5784)."""
    out = U128()
    rc = library().qpeps_known_count(int(n), ctypes.byref(out))
    return None if rc != QPEPS_OK else out.value


def certify_c(entries: Sequence[tuple[int, int]]) -> None:
    """Run the library's CompiledRowOperator::compile check on (legs_key, value) entries."""
    lib = library()
    m = len(entries)
    legs = (ctypes.c_uint32 * max(m, 1))(*[e[0] for e in entries])
    vals = (ctypes.c_uint64 * max(m, 1))(*[e[1] for e in entries])
    err = ctypes.create_string_buffer(4096)
    _check(lib.qpeps_certify_c(legs, vals, m, err, len(err)), err)


def version() -> str:
    return library().qpeps_version().decode()


def build() -> Path:
    """Compile libqpeps.so (sm_103a) in-tree; see buildlib.py."""
    import importlib  # noqa: PLC0415

    return importlib.import_module(__name__ + ".buildlib").build()
