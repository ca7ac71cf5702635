"""ctypes binding of the C oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker.  Restates the reference's parse path on the CPU (see cj_oracle.h).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import build as _build

ERR_UTF8 = 1
ERR_BRACKETS = 2
ERR_CAPACITY = 4


class _Stats(ctypes.Structure):
    _fields_ = [("n_structural", ctypes.c_int64), ("n_brackets", ctypes.c_int64),
                ("n_opens", ctypes.c_int64), ("max_depth", ctypes.c_int32),
                ("flags", ctypes.c_uint32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(str(path))
        L.cjo_parse.restype = ctypes.c_uint32
        L.cjo_parse.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                ctypes.POINTER(_Stats)]
        L.cjo_utf8_valid.restype = ctypes.c_int
        L.cjo_utf8_valid.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        L.cjo_query_lines.restype = ctypes.c_int64
        L.cjo_query_lines.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p,
                                      ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]
        L.cjo_utf8_refcompat.restype = ctypes.c_int
        L.cjo_utf8_refcompat.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        _lib = L
    return _lib


@dataclass
class OracleResult:
    positions: np.ndarray     # int32[S], 1-based byte offsets
    pair_row: np.ndarray      # int32[S], 1-based close index at opens, 0 elsewhere
    n_structural: int
    n_brackets: int
    n_opens: int
    max_depth: int
    flags: int

    @property
    def valid(self) -> bool:
        return self.flags == 0

    def reference_layout(self) -> np.ndarray:
        """The reference's result buffer: 2*(S+2) int32 (see cujson_gb300.h)."""
        S = self.n_structural
        out = np.zeros(2 * S + 4, dtype=np.int32)
        out[1:S + 1] = self.positions
        out[S + 1] = S + 1
        out[S + 2:2 * S + 2] = self.pair_row
        return out


def _as_u8(data) -> np.ndarray:
    if isinstance(data, (bytes, bytearray, memoryview)):
        return np.frombuffer(bytes(data), dtype=np.uint8)
    return np.ascontiguousarray(data, dtype=np.uint8)


def parse(data, lines: bool = False, chunk_sizes: Optional[Sequence[int]] = None) -> OracleResult:
    buf = _as_u8(data)
    n = buf.size
    cap = n + 1
    pos = np.zeros(cap, dtype=np.int32)
    pair = np.zeros(cap, dtype=np.int32)
    st = _Stats()
    cs = None
    ncs = 0
    if chunk_sizes is not None:
        cs = np.ascontiguousarray(np.asarray(chunk_sizes, dtype=np.uint64))
        ncs = cs.size
    lib().cjo_parse(buf.ctypes.data if n else None, n, int(lines),
                    cs.ctypes.data if cs is not None else None, ncs,
                    pos.ctypes.data, pair.ctypes.data, cap, ctypes.byref(st))
    S = st.n_structural
    return OracleResult(pos[:S].copy(), pair[:S].copy(), S, st.n_brackets, st.n_opens,
                        st.max_depth, st.flags)


def utf8_valid(data) -> bool:
    buf = _as_u8(data)
    return bool(lib().cjo_utf8_valid(buf.ctypes.data if buf.size else None, buf.size))


def utf8_refcompat(data) -> bool:
    buf = _as_u8(data)
    return bool(lib().cjo_utf8_refcompat(buf.ctypes.data if buf.size else None, buf.size))


def query_lines(data, res: OracleResult, key: bytes, value: Optional[bytes] = None, cap: int = 0):
    """The reference's record loop (gotoArrayIndex(0), checkKeyValue / findKey +
    getValue, gotoNextSibling(1)) over a JSON-Lines result: the count of
    matching records and, with `cap`, int64[min(count, cap), 3] of (record byte
    offset, value byte offset, value length) in visiting order."""
    buf = _as_u8(data)
    out = np.zeros((max(cap, 1), 3), np.int64)
    pos = np.ascontiguousarray(res.positions, np.int32)
    pair = np.ascontiguousarray(res.pair_row, np.int32)
    n = lib().cjo_query_lines(buf.ctypes.data if buf.size else None, buf.size, pos.ctypes.data, pair.ctypes.data,
                              res.n_structural, key, len(key), value or b"", len(value or b""),
                              int(value is not None), out.ctypes.data if cap else None, cap)
    return int(n), out[:min(int(n), cap)]
