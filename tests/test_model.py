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
from tests import synth  # noqa: E402  (seeded inputs)


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


def test_classify_bit_planes(model):
    """The bit-sliced character classes equal their byte-by-byte definition."""
    model.cjm_classify_check.restype = ctypes.c_int
    model.cjm_classify_check.argtypes = [ctypes.c_uint64, ctypes.c_int]
    assert model.cjm_classify_check(7, 20000) == 0


@pytest.mark.parametrize("seed", range(6))
def test_documents(cj, oracle, model, seed):
    n = [3000, 70000, 300000, 1 << 20, 123457, 9000][seed]
    d = synth.synth_document(1000 + seed, n, max_depth=8)
    check(model, oracle, d, seed=seed)


def test_huge_strings(cj, oracle, model):
    d = synth.synth_document(77, 3 << 20, max_depth=20, huge_string_frac=0.05,
                          huge_string_min=20000, huge_string_max=70000)
    check(model, oracle, d)


def test_backslash_runs(cj, oracle, model):
    for seed in range(4):
        check(model, oracle, synth.synth_backslash_string(seed, 100000 + seed * 777))


@pytest.mark.parametrize("depth", [1, 300, 5000, 20000])
def test_deep(cj, oracle, model, depth):
    check(model, oracle, synth.synth_deep(depth))


def test_lines(cj, oracle, model):
    d, _ = synth.synth_lines(5, 600000)
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
        d = synth.synth_document(42 + kind, 50000)
        assert synth.synth_corrupt(d, kind, kind)
        check(model, oracle, d)


def _utf8_soup(rng, n):
    """Mostly well-formed UTF-8 with sprinkled defects, as raw bytes."""
    out = bytearray()
    pieces = ["a", " ", "é", "€", "😀", "ߺ", "ࠀ", "￿", "\U00010000", "\U0010ffff", "퟿"]
    bad = [b"\xc0\x80", b"\xc1\xbf", b"\xe0\x80\x80", b"\xe0\x9f\xbf", b"\xed\xa0\x80", b"\xed\xbf\xbf",
           b"\xf0\x80\x80\x80", b"\xf0\x8f\xbf\xbf", b"\xf4\x90\x80\x80", b"\xf5\x80\x80\x80", b"\xff",
           b"\x80", b"\xbf", b"\xc3", b"\xe2\x82", b"\xf0\x9f\x98", b"\xc3\x41", b"\xe2\x41\x82"]
    while len(out) < n:
        if rng.random() < 0.02:
            out += bad[int(rng.integers(len(bad)))]
        else:
            out += pieces[int(rng.integers(len(pieces)))].encode("utf-8", "surrogatepass")
    return bytes(out[:n])


@pytest.mark.parametrize("seed", range(60))
def test_utf8_fuzz(oracle, model, seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(1, 3000)) if seed < 40 else int(rng.integers(120000, 140000))
    body = _utf8_soup(rng, n)
    if seed % 3 == 0:
        # sometimes cut the soup so the input ends inside a sequence
        body = body[: max(1, len(body) - int(rng.integers(0, 3)))]
    doc = b'["' + body.replace(b'"', b'x').replace(b'\\', b'x') + b'"]'
    p, q, fl = run_model(model, doc)
    assert bool(fl & 1) == (not oracle.utf8_valid(doc)), seed


def test_utf8_dense_short(oracle, model):
    # dense high bytes: every lead/continuation/invalid byte pattern near word,
    # lane and input-end boundaries
    rng = np.random.default_rng(77)
    vals = np.array(list(range(0x80, 0x100)) + [0x41, 0x20], dtype=np.uint8)
    for i in range(1500):
        n = int(rng.integers(1, 14))
        body = bytes(vals[rng.integers(0, vals.size, n)])
        pad = int(rng.integers(0, 40))
        doc = b"[" + b" " * pad + b'"' + body + b'"]'
        _, _, fl = run_model(model, doc)
        assert bool(fl & 1) == (not oracle.utf8_valid(doc)), (body, pad)
        doc2 = b'[""]' + b" " * pad + body        # the bytes end the input
        _, _, fl = run_model(model, doc2)
        assert bool(fl & 1) == (not oracle.utf8_valid(doc2)), (body, pad)


def test_utf8_across_region_and_tile_boundaries(oracle, model):
    """Multi-byte sequences, valid and invalid, placed across 32-byte lane,
    7 KiB warp-region and 112 KiB tile boundaries: the carries that hand an
    open sequence to the next lane, step or region."""
    seqs = ["é".encode(), "€".encode(), "😀".encode(), b"\xc0\x80", b"\xe0\x80\x80", b"\xed\xa0\x80",
            b"\xf0\x80\x80\x80", b"\xf4\x90\x80\x80", b"\xf5\x80\x80\x80", b"\xe2\x82", b"\x80", b"\xc3\x41",
            b"\xe0\xa0\x80", b"\xed\x9f\xbf", b"\xf0\x90\x80\x80", b"\xf4\x8f\xbf\xbf"]
    for boundary in (32, 1024, 7168, 114688):
        for body in seqs:
            for shift in range(-4, 2):
                pad = boundary + shift - 2          # the sequence starts at byte boundary + shift
                if pad < 0:
                    continue
                doc = b"[" + b" " * pad + b'"' + body + b'"]'
                _, _, fl = run_model(model, doc)
                assert bool(fl & 1) == (not oracle.utf8_valid(doc)), (boundary, body, shift)
                doc2 = b"[]" + b" " * (pad + 2) + body       # the sequence ends the input
                _, _, fl = run_model(model, doc2)
                assert bool(fl & 1) == (not oracle.utf8_valid(doc2)), (boundary, body, shift, "end")
