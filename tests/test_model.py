"""The kernels' algorithm, run sequentially on the CPU (tests/model/cj_model.cpp),
against the oracle: tiles, look-back composition, bracket levels and the
chunk/spine pairing, on seeded documents and adversarial inputs.  No GPU."""
import ctypes
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "model"))
import build as model_build  # noqa: E402


@pytest.fixture(scope="module")
def model():
    L = ctypes.CDLL(str(model_build.build()))
    L.cjm_parse.restype = ctypes.c_int
    L.cjm_parse.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                            ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                            ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint32),
                            ctypes.c_uint64]
    return L


def run_model(model, data, lines=False, chunks=None, seed=1):
    buf = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8) if isinstance(data, bytes) else data)
    cap = buf.size + 1
    pos = np.zeros(cap, np.int32)
    pair = np.zeros(cap, np.int32)
    S = ctypes.c_int64()
    fl = ctypes.c_uint32()
    cs = None
    if chunks is not None:
        cs = np.asarray(chunks, dtype=np.uint64)
    model.cjm_parse(buf.ctypes.data, buf.size, int(lines), cs.ctypes.data if cs is not None else None,
                    0 if cs is None else cs.size, pos.ctypes.data, pair.ctypes.data, cap,
                    ctypes.byref(S), ctypes.byref(fl), seed)
    return pos[:S.value], pair[:S.value], fl.value


def check(model, oracle, data, lines=False, chunks=None, seed=1):
    p, q, fl = run_model(model, data, lines, chunks, seed)
    r = oracle.parse(data, lines=lines, chunk_sizes=chunks)
    assert fl & 0xF00 == 0, hex(fl)          # internal consistency of the model
    assert bool(fl & 1) == bool(r.flags & oracle.ERR_UTF8)
    assert bool(fl & 2) == bool(r.flags & oracle.ERR_BRACKETS)
    np.testing.assert_array_equal(p, r.positions)
    if r.flags == 0:
        np.testing.assert_array_equal(q, r.pair_row)


@pytest.mark.parametrize("seed", range(6))
def test_documents(cj, oracle, model, seed):
    n = [3000, 70000, 300000, 1 << 20, 123457, 9000][seed]
    d = cj.synth_document(1000 + seed, n, max_depth=8)
    check(model, oracle, d, seed=seed)


def test_huge_strings(cj, oracle, model):
    d = cj.synth_document(77, 3 << 20, max_depth=20, huge_string_frac=0.05,
                          huge_string_min=20000, huge_string_max=70000)
    check(model, oracle, d)


def test_backslash_runs(cj, oracle, model):
    for seed in range(4):
        check(model, oracle, cj.synth_backslash_string(seed, 100000 + seed * 777))


@pytest.mark.parametrize("depth", [1, 300, 5000, 20000])
def test_deep(cj, oracle, model, depth):
    check(model, oracle, cj.synth_deep(depth))


def test_lines(cj, oracle, model):
    d, _ = cj.synth_lines(5, 600000)
    check(model, oracle, d, lines=True)
    # reference-style line-aligned chunks
    nl = np.flatnonzero(d == 10)
    cuts = [0, int(nl[len(nl) // 3]) + 1, int(nl[2 * len(nl) // 3]) + 1, d.size]
    check(model, oracle, d, lines=True, chunks=[cuts[i + 1] - cuts[i] for i in range(3)])


@pytest.mark.parametrize("seed", range(40))
def test_random_bytes(cj, oracle, model, seed):
    rng = np.random.default_rng(seed)
    alphabet = np.frombuffer(b'[]{}:,"\\ ab\n', np.uint8)
    n = int(rng.integers(1, 40000)) if seed < 30 else int(rng.integers(130000, 400000))
    d = alphabet[rng.integers(0, alphabet.size, n)]
    check(model, oracle, d, lines=bool(seed & 1))


def test_corrupt(cj, oracle, model):
    for kind in range(1, 6):
        d = cj.synth_document(42 + kind, 50000)
        assert cj.synth_corrupt(d, kind, kind)
        check(model, oracle, d)
