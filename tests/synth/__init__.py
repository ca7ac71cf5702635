"""Seeded synthetic inputs for the tests and the benchmark (ctypes view of
tests/synth/_build/libcj_synth.so, see cj_synth.h).

The reference is evaluated on ~1 GB real-world datasets that are not
available offline; these generators stand in for them with the shapes of the
benchmark configurations.  Not part of the parser library: nothing under
cujson_gb300/ loads this module.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import build as _build

# seeds of the benchmark configurations: CONFIG_SEED_BASE + configuration number
CONFIG_SEED_BASE = 0xC0DE0000
# largest JSON-Lines input (int32 positions, as in the reference)
LINES_CONFIG_BYTES = 2147483646


class SynthParams(ctypes.Structure):
    _fields_ = [("max_depth", ctypes.c_int32), ("keys_min", ctypes.c_int32),
                ("keys_max", ctypes.c_int32), ("nested_max_items", ctypes.c_int32),
                ("str_min", ctypes.c_int32), ("str_max", ctypes.c_int32),
                ("huge_string_frac", ctypes.c_double), ("huge_string_min", ctypes.c_int64),
                ("huge_string_max", ctypes.c_int64), ("block_bytes", ctypes.c_uint64),
                ("record_median", ctypes.c_double), ("record_sigma", ctypes.c_double),
                ("record_min", ctypes.c_int64), ("record_max", ctypes.c_int64),
                ("threads", ctypes.c_uint32)]


_SIGNATURES = {
    "cj_synth_default_params": (None, [ctypes.POINTER(SynthParams)]),
    "cj_synth_document": (ctypes.c_size_t, [ctypes.c_uint64, ctypes.c_size_t,
                                            ctypes.POINTER(SynthParams), ctypes.c_void_p]),
    "cj_synth_events": (ctypes.c_size_t, [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "cj_synth_lines": (ctypes.c_size_t, [ctypes.c_uint64, ctypes.c_size_t, ctypes.POINTER(SynthParams),
                                         ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "cj_synth_deep": (ctypes.c_size_t, [ctypes.c_size_t, ctypes.c_void_p]),
    "cj_synth_backslash_string": (ctypes.c_size_t, [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p]),
    "cj_synth_corrupt": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint64]),
}

_lib: Optional[ctypes.CDLL] = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        l = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


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


def synth_document_into(seed: int, out: np.ndarray, **kw) -> None:
    """synth_document written into a contiguous uint8 view (a slice of a batch buffer)."""
    if out.dtype != np.uint8 or not out.flags["C_CONTIGUOUS"]:
        raise ValueError("out must be a contiguous uint8 array")
    p = synth_params(**kw)
    n = lib().cj_synth_document(seed, out.size, ctypes.byref(p), out.ctypes.data)
    if n != out.size:
        raise ValueError("synth_document failed")


def synth_lines(seed: int, size: int, **kw):
    out = np.empty(size, dtype=np.uint8)
    p = synth_params(**kw)
    nrec = ctypes.c_uint64()
    n = lib().cj_synth_lines(seed, size, ctypes.byref(p), out.ctypes.data, ctypes.byref(nrec))
    if n != size:
        raise ValueError("synth_lines failed")
    return out, int(nrec.value)


def synth_events(seed: int, size: int):
    """Event-log JSON Lines of exactly `size` bytes: (bytes, records, PushEvent records)."""
    out = np.empty(size, dtype=np.uint8)
    nrec, npush = ctypes.c_uint64(), ctypes.c_uint64()
    n = lib().cj_synth_events(seed, size, out.ctypes.data, ctypes.byref(nrec), ctypes.byref(npush))
    if n != size:
        raise ValueError("synth_events failed")
    return out, int(nrec.value), int(npush.value)


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


# corruption kinds of cj_synth_corrupt
CORRUPT_OVERLONG2, CORRUPT_OVERLONG3, CORRUPT_SURROGATE, CORRUPT_UNBALANCED, CORRUPT_MISMATCHED = 1, 2, 3, 4, 5


def batch_input(seed: int, n_docs: int, total_bytes: int, min_size: int = 1 << 10,
                max_size: int = 16 << 20, sigma: float = 2.0, invalid_utf8: float = 0.01,
                invalid_brackets: float = 0.01, out: Optional[np.ndarray] = None):
    """A seeded batch of independent standard documents, back to back.

    Sizes are lognormal (sigma `sigma`), clamped to [min_size, max_size] and
    scaled so that they sum to about `total_bytes`.  A fraction of the
    documents gets an invalid UTF-8 sequence (overlong C0 80 / E0 80 80 or a
    surrogate ED A0 80 inside a string) and another fraction an unbalanced or
    mismatched bracket.  Returns (packed uint8 array, sizes int64[n],
    kinds int32[n]) where kinds[i] is 0 or the cj_synth_corrupt kind applied.
    `out` (>= the returned size, e.g. pinned) receives the documents if given.
    """
    rng = np.random.default_rng(seed)
    raw = rng.lognormal(mean=0.0, sigma=sigma, size=n_docs)
    sizes = raw * (total_bytes / raw.sum())
    for _ in range(8):   # re-scale after clamping
        sizes = np.clip(sizes, min_size, max_size)
        sizes *= total_bytes / sizes.sum()
    sizes = np.clip(np.round(sizes), min_size, max_size).astype(np.int64)
    total = int(sizes.sum())
    packed = out[:total] if out is not None else np.empty(total, np.uint8)
    kinds = np.zeros(n_docs, np.int32)
    n_utf = int(round(invalid_utf8 * n_docs))
    n_brk = int(round(invalid_brackets * n_docs))
    pick = rng.permutation(n_docs)
    for j, i in enumerate(pick[:n_utf]):
        kinds[i] = (CORRUPT_OVERLONG2, CORRUPT_OVERLONG3, CORRUPT_SURROGATE)[j % 3]
    for j, i in enumerate(pick[n_utf:n_utf + n_brk]):
        kinds[i] = (CORRUPT_UNBALANCED, CORRUPT_MISMATCHED)[j % 2]
    offs = np.concatenate([[0], np.cumsum(sizes)])

    def make(i):
        view = packed[int(offs[i]):int(offs[i + 1])]
        synth_document_into(seed * 1000003 + i, view, max_depth=8, threads=1)
        if kinds[i] and not synth_corrupt(view, int(kinds[i]), seed + i):
            kinds[i] = 0

    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        list(ex.map(make, range(n_docs)))
    return packed, sizes, kinds


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
        n = size or LINES_CONFIG_BYTES
        data, nrec = synth_lines(seed, n, max_depth=4)
        return data, {"kind": "lines", "records": nrec}
    raise ValueError(f"no single-input generator for config {config}")


def serve_requests(seed: int, n: int, median: int = 64 << 10, sigma: float = 1.6,
                   min_size: int = 256, max_size: int = 64 << 20, lines_frac: float = 0.2,
                   adversarial_frac: float = 0.005, deep_depth: int = 10000,
                   backslash_bytes: int = 32 << 20):
    """Seeded request pool: lognormal sizes (median `median`, tail clamped to
    `max_size`), `lines_frac` JSON-Lines documents, and `adversarial_frac`
    adversarial documents, alternately a `deep_depth`-deep [[...]] nesting and
    one string of `backslash_bytes` of backslash runs.  Returns (list of uint8
    arrays, lines flags bool[n], kinds: 0 standard, 1 JSON Lines, 2 deep,
    3 backslash string)."""
    rng = np.random.default_rng(seed)
    sizes = np.clip(np.round(median * rng.lognormal(0.0, sigma, n)), min_size, max_size).astype(np.int64)
    kinds = np.where(rng.random(n) < lines_frac, 1, 0)
    n_adv = int(round(adversarial_frac * n))
    adv = rng.choice(n, size=n_adv, replace=False) if n_adv else []
    for j, i in enumerate(adv):
        kinds[i] = 2 + (j % 2)
    docs = [None] * n

    def make(i):
        k = int(kinds[i])
        if k == 0:
            docs[i] = synth_document(seed * 7919 + i, int(sizes[i]), max_depth=8, threads=1)
        elif k == 1:
            docs[i] = synth_lines(seed * 7919 + i, int(sizes[i]), threads=1)[0]
        elif k == 2:
            docs[i] = synth_deep(deep_depth)
        else:
            docs[i] = synth_backslash_string(seed + i, backslash_bytes)

    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        list(ex.map(make, range(n)))
    return docs, kinds == 1, kinds


