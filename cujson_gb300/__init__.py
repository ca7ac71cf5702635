"""cujson_gb300 -- GB300-native (sm_103a) cuJSON parse path.

Python view of the C ABI in ``include/cujson_gb300.h`` (ctypes), used by the
tests and the benchmark.  The product is the shared library
``cujson_gb300/_build/libcujson_gb300.so``; C++ users include the drop-in
headers ``include/cujson/cujson.h`` / ``cujsonlines.h`` instead.

The entry points mirror the reference's parse interface:
``parse_standard_json(data)`` <- ``cuJSONResult parse_standard_json(cuJSONInput)``
(cujson/parse_standard_json.cu:1584) and ``parse_json_lines(chunks)`` <-
``cuJSONResult parse_json_lines(cuJSONLinesInput)`` (cujson/parse_json_lines.cu:1092),
with the same result layout.  There is no CPU fallback: if the library is not
built, or no GPU is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libcujson_gb300.so"

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_INVALID_UTF8 = 2
ERR_INVALID_BRACKETS = 3
ERR_TOO_LARGE = 4
ERR_OUT_OF_MEMORY = 5
ERR_CUDA = 6
ERR_TIMEOUT = 7
ERR_NO_DEVICE = 8
ERR_CAPACITY = 9
ERR_NOT_STAGED = 10

FLAG_UTF8 = 0x01
FLAG_BRACKETS = 0x02
FLAG_TIMEOUT = 0x04

MAX_INPUT_BYTES = 2147483646


class CujsonError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status) if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


class ParseInfo(ctypes.Structure):
    _fields_ = [("n_structural", ctypes.c_int64), ("n_brackets", ctypes.c_int64),
                ("max_depth", ctypes.c_int32), ("status", ctypes.c_int32),
                ("error_flags", ctypes.c_uint32), ("n_segments", ctypes.c_int32)]


class _Result(ctypes.Structure):
    _fields_ = [("structural", ctypes.POINTER(ctypes.c_int32)),
                ("pair_pos", ctypes.POINTER(ctypes.c_int32)),
                ("n_structural", ctypes.c_int64), ("total", ctypes.c_int64),
                ("max_depth", ctypes.c_int32), ("status", ctypes.c_int32),
                ("n_segments", ctypes.c_int64),
                ("segment_sizes", ctypes.POINTER(ctypes.c_int64))]


class ValueCounts(ctypes.Structure):
    """cj_value_counts: slots, and slots of each CJ_VAL_* type."""
    _fields_ = [("n_slots", ctypes.c_int64), ("by_type", ctypes.c_int64 * 8)]


VAL_NONE, VAL_STRING, VAL_INT, VAL_DOUBLE, VAL_TRUE, VAL_FALSE, VAL_NULL, VAL_INVALID = range(8)


class Tuning(ctypes.Structure):
    """Launch shapes (cj_tuning): 0 = default."""
    _fields_ = [("region_kib", ctypes.c_int32), ("scan_blocks_per_sm", ctypes.c_int32),
                ("emit_blocks_per_sm", ctypes.c_int32), ("pair_blocks", ctypes.c_int32),
                ("pair_threads", ctypes.c_int32), ("prefetch_steps", ctypes.c_int32),
                ("stream_wave_mib", ctypes.c_int32), ("ms", ctypes.c_float)]

    def as_dict(self):
        return {"region_kib": self.region_kib, "scan_blocks_per_sm": self.scan_blocks_per_sm,
                "emit_blocks_per_sm": self.emit_blocks_per_sm, "pair_blocks": self.pair_blocks,
                "pair_threads": self.pair_threads, "prefetch_steps": self.prefetch_steps,
                "stream_wave_mib": self.stream_wave_mib, "ms": round(float(self.ms), 4)}


_lib: Optional[ctypes.CDLL] = None

# name -> (restype, argtypes); the complete list of C-ABI exports
_SIGNATURES = {
    "cj_context_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "cj_context_destroy": (None, [ctypes.c_void_p]),
    "cj_context_reserve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]),
    "cj_context_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "cj_context_launch_count": (ctypes.c_int64, [ctypes.c_void_p]),
    "cj_context_device_bytes": (ctypes.c_size_t, [ctypes.c_void_p]),
    "cj_default_context": (ctypes.c_void_p, []),
    "cj_parse_standard": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                         ctypes.POINTER(_Result)]),
    "cj_parse_lines": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_size_t, ctypes.POINTER(_Result)]),
    "cj_parse_lines_planned": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                              ctypes.c_size_t, ctypes.POINTER(_Result)]),
    "cj_result_free": (None, [ctypes.POINTER(_Result)]),
    "cj_parse_into": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ParseInfo)]),
    "cj_parse_standard_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                                 ctypes.c_size_t, ctypes.POINTER(ParseInfo), ctypes.c_void_p]),
    "cj_stage_standard": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "cj_stage_lines": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_size_t]),
    "cj_run_staged": (ctypes.c_int, [ctypes.c_void_p]),
    "cj_run_staged_graph": (ctypes.c_int, [ctypes.c_void_p]),
    "cj_batch_padded_offsets": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                               ctypes.POINTER(ctypes.c_size_t)]),
    "cj_parse_batch_padded": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                             ctypes.c_int]),
    "cj_query_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p,
                                      ctypes.c_size_t, ctypes.POINTER(ctypes.c_int64)]),
    "cj_query_values": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p,
                                       ctypes.c_size_t, ctypes.POINTER(ctypes.c_int64)]),
    "cj_run_staged_starved": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ParseInfo)]),
    "cj_server_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "cj_server_destroy": (None, [ctypes.c_void_p]),
    "cj_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_uint64)]),
    "cj_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p,
                                      ctypes.POINTER(ctypes.c_double)]),
    "cj_server_take": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t]),
    "cj_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "cj_server_replay": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_double)]),
    "cj_stage_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                      ctypes.c_int]),
    "cj_stage_batch_packed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                             ctypes.c_int]),
    "cj_batch_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_size_t]),
    "cj_copy_batch_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "cj_context_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "cj_context_get_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "cj_autotune_staged": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "cj_staged_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ParseInfo)]),
    "cj_copy_staged_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "cj_staged_device_outputs": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                                ctypes.POINTER(ctypes.c_void_p)]),
    "cj_context_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cj_context_set_dependent_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cj_context_phase_ms": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_int64)]),
    "cj_context_scan_phase_ms": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_int64)]),
    "cj_context_span_ms": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "cj_host_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "cj_host_free": (None, [ctypes.c_void_p]),
    "cj_host_pool_trim": (ctypes.c_size_t, []),
    "cj_load_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p),
                                    ctypes.POINTER(ctypes.c_size_t)]),
    "cj_plan_lines_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                           ctypes.c_void_p]),
    "cj_plan_lines_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                           ctypes.c_void_p, ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_size_t)]),
    "cj_plan_lines_count_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                  ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    "cj_plan_lines_bytes_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                  ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                                  ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p]),
    "cj_decode_values": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "cj_context_staged_bytes": (ctypes.c_size_t, [ctypes.c_void_p]),
    "cj_values_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "cj_copy_values": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]),
    "cj_tuning_save": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "cj_tuning_load": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "cj_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "cj_last_status": (ctypes.c_int, []),
    "cj_last_error": (ctypes.c_char_p, []),
    "cj_set_last_status": (None, [ctypes.c_int]),
}


def exported_names() -> List[str]:
    return list(_SIGNATURES)


def lib() -> ctypes.CDLL:
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run cujson_gb300.build.build() first")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def status_string(status: int) -> str:
    return lib().cj_status_string(int(status)).decode()


def _check(st: int, what: str = "") -> None:
    if st != OK:
        raise CujsonError(st, what)


def _u8(data) -> np.ndarray:
    if isinstance(data, (bytes, bytearray, memoryview)):
        return np.frombuffer(bytes(data), dtype=np.uint8)
    return np.ascontiguousarray(data, dtype=np.uint8)


# ---------------------------------------------------------------------------
@dataclass
class ParseResult:
    """Host copy of a parse result in the reference's layout."""
    buffer: np.ndarray                 # int32[2*(S+2)]
    n_structural: int
    max_depth: int
    segment_sizes: List[int] = field(default_factory=list)

    @property
    def structural(self) -> np.ndarray:   # [0]=0, [1..S] positions, [S+1]=S+1
        return self.buffer[: self.n_structural + 2]

    @property
    def pair_pos(self) -> np.ndarray:     # [0]=S+1, [i] = close index for opens
        return self.buffer[self.n_structural + 1: 2 * self.n_structural + 3]

    @property
    def positions(self) -> np.ndarray:    # structural[1..S]
        return self.buffer[1: self.n_structural + 1]

    @property
    def pair_row(self) -> np.ndarray:     # pair_pos[1..S]
        return self.buffer[self.n_structural + 2: 2 * self.n_structural + 2]


def _take_result(r: _Result) -> ParseResult:
    S = int(r.n_structural)
    n = 2 * S + 4
    buf = np.ctypeslib.as_array(r.structural, shape=(n,)).copy()
    segs = [int(r.segment_sizes[i]) for i in range(int(r.n_segments))]
    out = ParseResult(buf, S, int(r.max_depth), segs)
    lib().cj_result_free(ctypes.byref(r))
    return out


class Context:
    """One device, one stream, one reusable device arena."""

    def __init__(self, device: int = -1):
        h = ctypes.c_void_p()
        _check(lib().cj_context_create(device, ctypes.byref(h)), "cj_context_create")
        self._h = h

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            lib().cj_context_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def reserve(self, max_bytes: int, max_segments: int = 1) -> None:
        _check(lib().cj_context_reserve(self._h, max_bytes, max_segments), "reserve")

    @property
    def stream(self) -> int:
        return lib().cj_context_stream(self._h) or 0

    @property
    def launches(self) -> int:
        return int(lib().cj_context_launch_count(self._h))

    @property
    def device_bytes(self) -> int:
        return int(lib().cj_context_device_bytes(self._h))

    # ---- one-shot, reference-shaped ------------------------------------------
    def parse_standard_json(self, data) -> ParseResult:
        buf = _u8(data)
        r = _Result()
        st = lib().cj_parse_standard(self._h, buf.ctypes.data if buf.size else None, buf.size,
                                     ctypes.byref(r))
        _check(st, "parse_standard_json")
        return _take_result(r)

    def parse_json_lines(self, chunks: Sequence) -> ParseResult:
        arrs = [_u8(c) for c in chunks]
        ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data if a.size else None for a in arrs])
        sizes = (ctypes.c_size_t * len(arrs))(*[a.size for a in arrs])
        r = _Result()
        st = lib().cj_parse_lines(self._h, ptrs, sizes, len(arrs), ctypes.byref(r))
        _check(st, "parse_json_lines")
        return _take_result(r)

    def parse_lines_planned(self, data, chunk_count: int = 0, chunk_bytes: int = 0) -> ParseResult:
        """cj_parse_lines_planned: one JSON-Lines buffer, its chunks planned on
        the device (chunk_count != 0: by count; else by the byte limit)."""
        buf = _u8(data)
        r = _Result()
        st = lib().cj_parse_lines_planned(self._h, buf.ctypes.data if buf.size else None, buf.size, chunk_count,
                                          chunk_bytes, ctypes.byref(r))
        _check(st, "parse_lines_planned")
        return _take_result(r)

    def try_parse(self, data, lines: bool = False, chunk_sizes: Optional[Sequence[int]] = None):
        """(status, ParseResult or None) without raising on invalid input."""
        buf = _u8(data)
        r = _Result()
        if lines:
            sizes_l = list(chunk_sizes) if chunk_sizes is not None else [buf.size]
            offs = np.cumsum([0] + sizes_l[:-1])
            ptrs = (ctypes.c_void_p * len(sizes_l))(*[buf.ctypes.data + int(o) for o in offs])
            sizes = (ctypes.c_size_t * len(sizes_l))(*sizes_l)
            st = lib().cj_parse_lines(self._h, ptrs, sizes, len(sizes_l), ctypes.byref(r))
        else:
            st = lib().cj_parse_standard(self._h, buf.ctypes.data if buf.size else None, buf.size,
                                         ctypes.byref(r))
        if st != OK:
            return st, None
        return st, _take_result(r)

    # ---- staged device-resident runs --------------------------------------------
    def stage_standard(self, data) -> None:
        buf = _u8(data)
        _check(lib().cj_stage_standard(self._h, buf.ctypes.data, buf.size), "stage")

    def stage_lines(self, data, chunk_sizes: Sequence[int]) -> None:
        buf = _u8(data)
        offs = np.cumsum([0] + list(chunk_sizes)[:-1])
        ptrs = (ctypes.c_void_p * len(chunk_sizes))(*[buf.ctypes.data + int(o) for o in offs])
        sizes = (ctypes.c_size_t * len(chunk_sizes))(*chunk_sizes)
        _check(lib().cj_stage_lines(self._h, ptrs, sizes, len(chunk_sizes)), "stage_lines")

    def run(self) -> None:
        _check(lib().cj_run_staged(self._h), "run")

    def info(self) -> ParseInfo:
        inf = ParseInfo()
        _check(lib().cj_staged_info(self._h, ctypes.byref(inf)), "info")
        return inf

    def staged_result(self) -> ParseResult:
        inf = self.info()
        S = int(inf.n_structural)
        buf = np.zeros(2 * S + 4, dtype=np.int32)
        _check(lib().cj_copy_staged_result(self._h, buf.ctypes.data, buf.size), "copy")
        return ParseResult(buf, S, int(inf.max_depth))

    # ---- queries on the device over the staged JSON-Lines result --------------------
    def query_count(self, key: bytes, value: bytes) -> int:
        """Records whose `key` has the value `value` (checkKeyValue semantics)."""
        n = ctypes.c_int64()
        _check(lib().cj_query_count(self._h, key, len(key), value, len(value), ctypes.byref(n)), "query_count")
        return n.value

    def query_values(self, key: bytes, cap: Optional[int] = None) -> np.ndarray:
        """int64[m, 3]: record offset, value offset, value length, in document
        order, for the records that have `key`.  Without `cap`, a first pass
        counts them."""
        n = ctypes.c_int64()
        if cap is None:
            _check(lib().cj_query_values(self._h, key, len(key), None, 0, ctypes.byref(n)), "query_values")
            cap = n.value
        out = np.zeros((max(cap, 1), 3), np.int64)
        _check(lib().cj_query_values(self._h, key, len(key), out.ctypes.data if cap else None, cap,
                                     ctypes.byref(n)), "query_values")
        return out[: n.value]

    def run_graph(self) -> None:
        _check(lib().cj_run_staged_graph(self._h), "run_graph")

    # ---- batches of independent documents ------------------------------------------
    def stage_batch(self, docs: Sequence, lines: bool = False) -> None:
        """Stage documents given one buffer each (kept alive by the caller until
        this returns)."""
        bufs = [_u8(d) for d in docs]
        ptrs = (ctypes.c_void_p * len(bufs))(*[b.ctypes.data for b in bufs])
        sizes = (ctypes.c_size_t * len(bufs))(*[b.size for b in bufs])
        self._batch_n = len(bufs)
        _check(lib().cj_stage_batch(self._h, ptrs, sizes, len(bufs), int(lines)), "stage_batch")

    def stage_batch_packed(self, packed, sizes: Sequence[int], lines: bool = False) -> None:
        """Stage documents laid back to back in one buffer (pinned for speed)."""
        buf = _u8(packed)
        sz = np.ascontiguousarray(np.asarray(sizes, dtype=np.uint64))
        if int(sz.sum()) > buf.size:
            raise ValueError("sizes exceed the packed buffer")
        self._batch_n = int(sz.size)
        _check(lib().cj_stage_batch_packed(self._h, buf.ctypes.data, sz.ctypes.data, int(sz.size),
                                           int(lines)), "stage_batch_packed")

    def parse_batch_padded(self, padded, sizes: Sequence[int], lines: bool = False) -> None:
        """Parse documents laid out by batch_padded_offsets (pinned for the
        overlap of copy and parse); read results with batch_info / batch_layout."""
        buf = _u8(padded)
        sz = np.ascontiguousarray(np.asarray(sizes, dtype=np.uint64))
        self._batch_n = int(sz.size)
        _check(lib().cj_parse_batch_padded(self._h, buf.ctypes.data, sz.ctypes.data, int(sz.size), int(lines)),
               "parse_batch_padded")

    def batch_info(self):
        """(status int32[n], n_structural int64[n], max_depth int32[n], offsets int64[n+1])."""
        n = self._batch_n
        status = np.zeros(n, np.int32)
        S = np.zeros(n, np.int64)
        depth = np.zeros(n, np.int32)
        off = np.zeros(n + 1, np.int64)
        _check(lib().cj_batch_info(self._h, status.ctypes.data, S.ctypes.data, depth.ctypes.data,
                                   off.ctypes.data, n), "batch_info")
        return status, S, depth, off

    def batch_layout(self, out: Optional[np.ndarray] = None):
        """Every document's reference layout back to back, with the info arrays."""
        status, S, depth, off = self.batch_info()
        total = int(off[-1])
        if out is None or out.size < total:
            out = np.empty(total, np.int32)
        _check(lib().cj_copy_batch_result(self._h, out.ctypes.data, out.size), "copy_batch")
        return out, status, S, depth, off

    def batch_results(self):
        """List of (status, ParseResult or None) per document."""
        layout, status, S, depth, off = self.batch_layout()
        res = []
        for i in range(status.size):
            if status[i] != OK:
                res.append((int(status[i]), None))
            else:
                buf = layout[off[i]:off[i + 1]].copy()
                res.append((OK, ParseResult(buf, int(S[i]), int(depth[i]))))
        return res

    # ---- launch shapes -------------------------------------------------------------
    def set_tuning(self, region_kib: int = 0, scan_blocks_per_sm: int = 0, emit_blocks_per_sm: int = 0,
                   pair_blocks: int = 0, pair_threads: int = 0, prefetch_steps: int = 0,
                   stream_wave_mib: int = 0) -> None:
        t = Tuning(region_kib, scan_blocks_per_sm, emit_blocks_per_sm, pair_blocks, pair_threads,
                   prefetch_steps, stream_wave_mib, 0.0)
        _check(lib().cj_context_set_tuning(self._h, ctypes.byref(t)), "set_tuning")

    def get_tuning(self) -> Tuning:
        t = Tuning()
        _check(lib().cj_context_get_tuning(self._h, ctypes.byref(t)), "get_tuning")
        return t

    def decode_values(self):
        """cj_decode_values on the staged result, copied out: (types uint8[S+1],
        nums uint64[S+1], lens uint32[S+1], strings uint8[n_bytes], counts
        by type).  Slot 0 is the text before the first structural, slot i the
        text after structural i."""
        counts = ValueCounts()
        _check(lib().cj_decode_values(self._h, ctypes.byref(counts)), "decode_values")
        n = int(counts.n_slots)
        types = np.zeros(n, np.uint8)
        nums = np.zeros(n, np.uint64)
        lens = np.zeros(n, np.uint32)
        nbytes = int(lib().cj_context_staged_bytes(self._h))
        strings = np.zeros(max(1, nbytes), np.uint8)
        _check(lib().cj_copy_values(self._h, types.ctypes.data, nums.ctypes.data, lens.ctypes.data, n,
                                    strings.ctypes.data, strings.size), "copy_values")
        return types, nums, lens, strings, [int(x) for x in counts.by_type]

    def decode_values_counts(self) -> List[int]:
        """cj_decode_values on the staged result, leaving the arrays on the
        device: the slot counts by type."""
        counts = ValueCounts()
        _check(lib().cj_decode_values(self._h, ctypes.byref(counts)), "decode_values")
        return [int(x) for x in counts.by_type]

    def save_tuning(self, path: str) -> None:
        _check(lib().cj_tuning_save(self._h, str(path).encode()), "save_tuning")

    def load_tuning(self, path: str) -> None:
        _check(lib().cj_tuning_load(self._h, str(path).encode()), "load_tuning")

    def autotune(self, reps: int = 3):
        """Times graph replays of the staged input for each candidate launch
        shape and keeps the fastest; returns (best, [tried])."""
        best = Tuning()
        tried = (Tuning * 128)()
        n = ctypes.c_size_t()
        _check(lib().cj_autotune_staged(self._h, reps, ctypes.byref(best), tried, len(tried), ctypes.byref(n)),
               "autotune")
        return best, [tried[i] for i in range(min(n.value, len(tried)))]

    def set_dependent_launch(self, enable: bool) -> None:
        """cj_context_set_dependent_launch: whether the kernels after the first
        of a run are scheduled while the one before finishes (default on)."""
        _check(lib().cj_context_set_dependent_launch(self._h, int(bool(enable))), "set_dependent_launch")

    def timing(self, enable: int = 1) -> None:
        """cj_context_timing: 0 off; 1 (True) an event at every kernel
        boundary; 2 events at the run's start, the scan's end and the run's
        end only, so the scan's kernels overlap their launches as untimed runs
        do; 3 events at the run's start and end only."""
        _check(lib().cj_context_timing(self._h, int(enable)), "timing")

    def phase_ms(self):
        """(scan_ms, pair_ms, spine_ms, runs) summed over the recorded runs."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int64()
        _check(lib().cj_context_phase_ms(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                         ctypes.byref(n)), "phase_ms")
        return a.value, b.value, c.value, n.value

    def scan_phase_ms(self):
        """(tables_ms, prefix_ms, emit_ms, runs): the scan's kernels, summed over
        the recorded runs."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int64()
        _check(lib().cj_context_scan_phase_ms(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                              ctypes.byref(n)), "scan_phase_ms")
        return a.value, b.value, c.value, n.value

    def span_ms(self) -> float:
        v = ctypes.c_double()
        _check(lib().cj_context_span_ms(self._h, ctypes.byref(v)), "span_ms")
        return v.value

    def plan_lines_count_device(self, d_ptr: int, size: int, chunk_count: int, stream: int = 0) -> List[int]:
        """cj_plan_lines_count_device: the chunk plan of a JSON-Lines buffer at
        device address `d_ptr` (`size` bytes), computed on the device after the
        work queued so far on `stream` (a cudaStream_t handle; 0 = the legacy
        default stream), which is the stream that fills the buffer."""
        out = np.zeros(chunk_count, dtype=np.uint64)
        _check(lib().cj_plan_lines_count_device(self._h, ctypes.c_void_p(d_ptr) if size else None, size,
                                                chunk_count, out.ctypes.data,
                                                ctypes.c_void_p(stream) if stream else None),
               "plan_lines_count_device")
        return [int(x) for x in out]

    def plan_lines_bytes_device(self, d_ptr: int, size: int, chunk_bytes: int, stream: int = 0) -> List[int]:
        """cj_plan_lines_bytes_device: the byte-limit chunk plan of a JSON-Lines
        buffer at device address `d_ptr`, computed on the device (`stream` as
        for plan_lines_count_device)."""
        dp = ctypes.c_void_p(d_ptr) if size else None
        sp = ctypes.c_void_p(stream) if stream else None
        n = ctypes.c_size_t()
        _check(lib().cj_plan_lines_bytes_device(self._h, dp, size, chunk_bytes, None, 0, ctypes.byref(n), sp),
               "plan_lines_bytes_device")
        out = np.zeros(max(1, n.value), dtype=np.uint64)
        _check(lib().cj_plan_lines_bytes_device(self._h, dp, size, chunk_bytes, out.ctypes.data, out.size,
                                                ctypes.byref(n), sp), "plan_lines_bytes_device")
        return [int(x) for x in out[: n.value]]

    def parse_into(self, data, out: np.ndarray, lines: bool = False) -> ParseInfo:
        buf = _u8(data)
        inf = ParseInfo()
        st = lib().cj_parse_into(self._h, buf.ctypes.data, buf.size, int(lines), out.ctypes.data,
                                 out.size, ctypes.byref(inf))
        _check(st, "parse_into")
        return inf


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("slots", ctypes.c_uint32),
                ("max_batch_docs", ctypes.c_uint32), ("memory_budget", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_uint64), ("docs", ctypes.c_uint64), ("bytes", ctypes.c_uint64),
                ("max_batch_docs", ctypes.c_uint64), ("peak_admitted_bytes", ctypes.c_uint64),
                ("device_bytes", ctypes.c_uint64), ("fault", ctypes.c_int32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class Server:
    """Parse server with continuous batching (cj_server_*).  Submitted buffers
    must stay alive until their request completes; the server keeps a
    reference to each submitted array until it is taken."""

    def __init__(self, device: int = -1, slots: int = 2, max_batch_docs: int = 1024,
                 memory_budget: int = 16 << 30):
        cfg = ServerConfig(device, slots, max_batch_docs, memory_budget)
        h = ctypes.c_void_p()
        _check(lib().cj_server_create(ctypes.byref(cfg), ctypes.byref(h)), "cj_server_create")
        self._h = h
        self._keep = {}

    def close(self) -> None:
        if self._h:
            lib().cj_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, data, lines: bool = False) -> int:
        buf = _u8(data)
        t = ctypes.c_uint64()
        _check(lib().cj_server_submit(self._h, buf.ctypes.data, buf.size, int(lines), ctypes.byref(t)),
               "submit")
        self._keep[t.value] = buf
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(ParseInfo, latency seconds)."""
        inf = ParseInfo()
        lat = ctypes.c_double()
        _check(lib().cj_server_wait(self._h, ticket, timeout_ms, ctypes.byref(inf), ctypes.byref(lat)),
               "wait")
        return inf, lat.value

    def take(self, ticket: int):
        """(status, ParseResult or None) of a completed request; releases it."""
        inf, _ = self.wait(ticket)
        S = int(inf.n_structural)
        out = np.zeros(2 * S + 4, np.int32) if inf.status == OK else None
        st = lib().cj_server_take(self._h, ticket, out.ctypes.data if out is not None else None,
                                  out.size if out is not None else 0)
        self._keep.pop(ticket, None)
        if st != OK:
            return st, None
        return st, ParseResult(out, S, int(inf.max_depth))

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check(lib().cj_server_get_stats(self._h, ctypes.byref(st)), "stats")
        return st

    def replay(self, docs: Sequence, lines: Sequence[bool], arrival_s: Sequence[float]):
        """Submit docs[i] at arrival_s[i] (seconds from now), wait for all;
        returns (status int32[n], latency float64[n], makespan seconds)."""
        n = len(docs)
        bufs = [_u8(d) for d in docs]
        ptrs = (ctypes.c_void_p * n)(*[b.ctypes.data for b in bufs])
        sizes = np.ascontiguousarray([b.size for b in bufs], dtype=np.uint64)
        ln = np.ascontiguousarray(lines, dtype=np.int32)
        arr = np.ascontiguousarray(arrival_s, dtype=np.float64)
        status = np.zeros(n, np.int32)
        lat = np.zeros(n, np.float64)
        mk = ctypes.c_double()
        _check(lib().cj_server_replay(self._h, ptrs, sizes.ctypes.data, ln.ctypes.data, arr.ctypes.data, n,
                                      status.ctypes.data, lat.ctypes.data, ctypes.byref(mk)), "replay")
        return status, lat, mk.value


_default: Optional[Context] = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context()
    return _default


def parse_standard_json(data) -> ParseResult:
    return default_context().parse_standard_json(data)


def parse_json_lines(chunks: Sequence) -> ParseResult:
    return default_context().parse_json_lines(chunks)


class PinnedBuffer:
    """Pinned host memory viewed as a numpy array (freed on close / GC)."""

    def __init__(self, nbytes: int, dtype=np.uint8):
        self._p = lib().cj_host_alloc(max(1, nbytes))
        if not self._p:
            raise MemoryError("cj_host_alloc failed")
        n = nbytes // np.dtype(dtype).itemsize
        raw = (ctypes.c_uint8 * max(1, nbytes)).from_address(self._p)
        self.array = np.frombuffer(raw, dtype=np.uint8, count=n * np.dtype(dtype).itemsize).view(dtype)

    def close(self):
        if self._p:
            self.array = None
            lib().cj_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_lines_count(data, chunk_count: int) -> List[int]:
    buf = _u8(data)
    out = np.zeros(chunk_count, dtype=np.uint64)
    _check(lib().cj_plan_lines_count(buf.ctypes.data if buf.size else None, buf.size, chunk_count,
                                     out.ctypes.data), "plan_lines_count")
    return [int(x) for x in out]


def plan_lines_bytes(data, chunk_bytes: int) -> List[int]:
    buf = _u8(data)
    n = ctypes.c_size_t()
    _check(lib().cj_plan_lines_bytes(buf.ctypes.data if buf.size else None, buf.size, chunk_bytes,
                                     None, 0, ctypes.byref(n)), "plan_lines_bytes")
    out = np.zeros(max(1, n.value), dtype=np.uint64)
    _check(lib().cj_plan_lines_bytes(buf.ctypes.data if buf.size else None, buf.size, chunk_bytes,
                                     out.ctypes.data, out.size, ctypes.byref(n)), "plan_lines_bytes")
    return [int(x) for x in out[: n.value]]


def batch_padded_offsets(sizes: Sequence[int]):
    """(offsets uint64[n], total bytes): the 1 KiB-aligned layout of a batch."""
    sz = np.ascontiguousarray(np.asarray(sizes, dtype=np.uint64))
    off = np.zeros(max(1, sz.size), np.uint64)
    tot = ctypes.c_size_t()
    _check(lib().cj_batch_padded_offsets(sz.ctypes.data, sz.size, off.ctypes.data, ctypes.byref(tot)),
           "batch_padded_offsets")
    return off[:sz.size], int(tot.value)
