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


class SynthParams(ctypes.Structure):
    _fields_ = [("max_depth", ctypes.c_int32), ("keys_min", ctypes.c_int32),
                ("keys_max", ctypes.c_int32), ("nested_max_items", ctypes.c_int32),
                ("str_min", ctypes.c_int32), ("str_max", ctypes.c_int32),
                ("huge_string_frac", ctypes.c_double), ("huge_string_min", ctypes.c_int64),
                ("huge_string_max", ctypes.c_int64), ("block_bytes", ctypes.c_uint64),
                ("record_median", ctypes.c_double), ("record_sigma", ctypes.c_double),
                ("record_min", ctypes.c_int64), ("record_max", ctypes.c_int64),
                ("threads", ctypes.c_uint32)]


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
    "cj_result_free": (None, [ctypes.POINTER(_Result)]),
    "cj_parse_into": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ParseInfo)]),
    "cj_parse_standard_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                                 ctypes.c_size_t, ctypes.POINTER(ParseInfo), ctypes.c_void_p]),
    "cj_stage_standard": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "cj_stage_lines": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_size_t]),
    "cj_run_staged": (ctypes.c_int, [ctypes.c_void_p]),
    "cj_staged_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ParseInfo)]),
    "cj_copy_staged_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "cj_staged_device_outputs": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                                ctypes.POINTER(ctypes.c_void_p)]),
    "cj_context_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cj_context_phase_ms": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_int64)]),
    "cj_context_span_ms": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "cj_host_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "cj_host_free": (None, [ctypes.c_void_p]),
    "cj_load_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p),
                                    ctypes.POINTER(ctypes.c_size_t)]),
    "cj_plan_lines_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                           ctypes.c_void_p]),
    "cj_plan_lines_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                           ctypes.c_void_p, ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_size_t)]),
    "cj_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "cj_last_status": (ctypes.c_int, []),
    "cj_set_last_status": (None, [ctypes.c_int]),
    "cj_synth_default_params": (None, [ctypes.POINTER(SynthParams)]),
    "cj_synth_document": (ctypes.c_size_t, [ctypes.c_uint64, ctypes.c_size_t,
                                            ctypes.POINTER(SynthParams), ctypes.c_void_p]),
    "cj_synth_lines": (ctypes.c_size_t, [ctypes.c_uint64, ctypes.c_size_t, ctypes.POINTER(SynthParams),
                                         ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "cj_synth_deep": (ctypes.c_size_t, [ctypes.c_size_t, ctypes.c_void_p]),
    "cj_synth_backslash_string": (ctypes.c_size_t, [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p]),
    "cj_synth_corrupt": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint64]),
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

    def timing(self, enable: bool = True) -> None:
        _check(lib().cj_context_timing(self._h, int(enable)), "timing")

    def phase_ms(self):
        """(scan_ms, pair_ms, spine_ms, runs) summed over the recorded runs."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int64()
        _check(lib().cj_context_phase_ms(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                         ctypes.byref(n)), "phase_ms")
        return a.value, b.value, c.value, n.value

    def span_ms(self) -> float:
        v = ctypes.c_double()
        _check(lib().cj_context_span_ms(self._h, ctypes.byref(v)), "span_ms")
        return v.value

    def parse_into(self, data, out: np.ndarray, lines: bool = False) -> ParseInfo:
        buf = _u8(data)
        inf = ParseInfo()
        st = lib().cj_parse_into(self._h, buf.ctypes.data, buf.size, int(lines), out.ctypes.data,
                                 out.size, ctypes.byref(inf))
        _check(st, "parse_into")
        return inf


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


# ---------------------------------------------------------------------------
# seeded synthetic inputs (stand-ins for the reference's evaluation datasets)
CONFIG_SEED_BASE = 0xC0DE0000


def synth_params(**kw) -> SynthParams:
    p = SynthParams()
    lib().cj_synth_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def synth_document(seed: int, size: int, **kw) -> np.ndarray:
    out = np.empty(size, dtype=np.uint8)
    p = synth_params(**kw)
    n = lib().cj_synth_document(seed, size, ctypes.byref(p), out.ctypes.data)
    if n != size:
        raise ValueError("synth_document failed")
    return out


def synth_lines(seed: int, size: int, **kw):
    out = np.empty(size, dtype=np.uint8)
    p = synth_params(**kw)
    nrec = ctypes.c_uint64()
    n = lib().cj_synth_lines(seed, size, ctypes.byref(p), out.ctypes.data, ctypes.byref(nrec))
    if n != size:
        raise ValueError("synth_lines failed")
    return out, int(nrec.value)


def synth_deep(depth: int) -> np.ndarray:
    out = np.empty(2 * depth, dtype=np.uint8)
    lib().cj_synth_deep(depth, out.ctypes.data)
    return out


def synth_backslash_string(seed: int, body: int) -> np.ndarray:
    out = np.empty(body + 4, dtype=np.uint8)
    lib().cj_synth_backslash_string(seed, body, out.ctypes.data)
    return out


def synth_corrupt(doc: np.ndarray, kind: int, seed: int = 0) -> bool:
    return bool(lib().cj_synth_corrupt(doc.ctypes.data, doc.size, kind, seed))


def config_input(config: int, size: Optional[int] = None):
    """The seeded stand-in input of a benchmark configuration.

    1: standard JSON, 64 MiB, depth <= 6.
    2: standard JSON, 1 GiB, depth <= 20, 1% of strings 64-256 KiB of backslash runs.
    3: JSON Lines, 2,147,483,646 bytes, lognormal records (median 200 B, 50 B..2 KiB).
    Returns (bytes as uint8 array, info dict).
    """
    seed = CONFIG_SEED_BASE + config
    if config == 1:
        n = size or (64 << 20)
        return synth_document(seed, n, max_depth=6), {"kind": "standard", "max_depth": 6}
    if config == 2:
        n = size or (1 << 30)
        return (synth_document(seed, n, max_depth=20, huge_string_frac=0.01),
                {"kind": "standard", "max_depth": 20, "huge_string_frac": 0.01})
    if config == 3:
        n = size or MAX_INPUT_BYTES
        data, nrec = synth_lines(seed, n, max_depth=4)
        return data, {"kind": "lines", "records": nrec}
    raise ValueError(f"no single-input generator for config {config}")
