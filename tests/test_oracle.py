"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests and no golden outputs, so the oracle is pinned by
(a) hand-derived answers for small documents, worked out from the reference's
output contract (cujson/parse_standard_json.cu:1659-1680: 1-based positions,
pair indices at opens), (b) the structure counts of the reference's two
sample files, and (c) golden fixtures produced by the reference's own code
(tests/golden, checked in test_golden.py).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import build_ref

REF_DATASET = build_ref.DEFAULT_REF / "dataset"


def _pos(r):
    return r.positions.tolist()


def _pairs(r):
    return r.pair_row.tolist()


@pytest.mark.parametrize("doc,pos,pairs", [
    (b"[1,2]", [1, 3, 5], [3, 0, 0]),
    (b'{"a":"b\\"c,d"}', [1, 5, 14], [3, 0, 0]),
    (b'["\\\\",1]', [1, 6, 8], [3, 0, 0]),
    (b'["\\\\\\"",1]', [1, 8, 10], [3, 0, 0]),
    (b'{"k":[{},[]],"x":{}}', [1, 5, 6, 7, 8, 9, 10, 11, 12, 13, 17, 18, 19, 20],
     [14, 0, 9, 5, 0, 0, 8, 0, 0, 0, 0, 13, 0, 0]),
    (b'"[{,:}]"', [], []),
    (b"123", [], []),
    (b"   ", [], []),
    (b'[":" , "{" ]', [1, 6, 12], [3, 0, 0]),
])
def test_known_answers(oracle, doc, pos, pairs):
    r = oracle.parse(doc)
    assert r.flags == 0
    assert _pos(r) == pos
    assert _pairs(r) == pairs


def test_escapes_outside_strings_count(oracle):
    # backslashes escape the next byte wherever they are (the reference's
    # bitmap logic does not look at string state)
    r = oracle.parse(b'[\\"x",1]')
    # the quote at 2 is escaped, the one at 4 opens a string that never closes
    assert _pos(r) == [1]


def test_json_lines_chunks(oracle):
    doc = b'{"a":1}\n{"b":[2]}\n'
    r = oracle.parse(doc, lines=True)
    assert _pos(r) == [1, 5, 7, 8, 9, 13, 14, 16, 17, 18]
    assert _pairs(r) == [3, 0, 0, 0, 9, 0, 8, 0, 0, 0]
    # chunking changes nothing for whole records
    r2 = oracle.parse(doc, lines=True, chunk_sizes=[8, 11])
    assert _pos(r2) == _pos(r) and _pairs(r2) == _pairs(r)


def test_json_lines_chunk_state_restarts(oracle):
    # an unterminated string in chunk 1 does not leak into chunk 2
    doc = b'["x\n["y"]\n'
    r = oracle.parse(doc, lines=True, chunk_sizes=[4, 6])
    assert r.flags & oracle.ERR_BRACKETS          # chunk 1 has an unclosed '['
    assert _pos(r)[:1] == [1]
    assert 5 in _pos(r) and 9 in _pos(r)


@pytest.mark.parametrize("doc,ok", [
    ("é".encode(), True), ("€".encode(), True), ("😀".encode(), True),
    (b"\xc0\x80", False), (b"\xe0\x80\x80", False), (b"\xed\xa0\x80", False),
    (b"\xf5\x80\x80\x80", False), (b"\xe2\x82", False), (b"\x80", False),
    (b"\xc3\x41", False), (b"\xf4\x90\x80\x80", False), (b"\xf0\x80\x80\x80", False),
    (b"\xef\xbf\xbf", True), (b"\xf4\x8f\xbf\xbf", True), (b"\xc2\x80", True),
])
def test_utf8_strict(oracle, doc, ok):
    assert oracle.utf8_valid(doc) == ok
    r = oracle.parse(b'["' + doc + b'"]')
    assert bool(r.flags & oracle.ERR_UTF8) == (not ok)


@pytest.mark.parametrize("doc", [
    b"\xc0\x80AB", b"\xe0\x80\x80A", b"\xed\xa0\x80A", b"\xf5\x80\x80\x80", b"\xc3\x41AA",
    b"AAA\xe2",            # truncation at EOF
])
def test_refcompat_accepts_what_strict_rejects(oracle, doc):
    # defect 1 of the reference's validator: the first-byte classes are
    # overwritten (parse_standard_json.cu:122-123), so these pass
    assert oracle.utf8_refcompat(doc)
    assert not oracle.utf8_valid(doc)


def test_refcompat_rejects(oracle):
    # an incomplete lead at a word end followed by an all-ASCII word
    assert not oracle.utf8_refcompat(b"AAA\xe2AAAA")
    # valid text is accepted
    assert oracle.utf8_refcompat("aé€😀b".encode())


@pytest.mark.parametrize("doc", [b"[}", b"{]", b"[[]", b"[]]", b"][", b"}{{}", b"[{]}"])
def test_brackets_rejected(oracle, doc):
    assert oracle.parse(doc).flags & oracle.ERR_BRACKETS


@pytest.mark.skipif(not REF_DATASET.exists(), reason="reference dataset not mounted")
@pytest.mark.parametrize("name,S,opens", [
    ("twitter_sample_large_record.json", 22388, 1769),
    ("twitter_sample_small_records.json", 22336, 1768),
])
def test_reference_samples(oracle, name, S, opens):
    data = (REF_DATASET / name).read_bytes()
    lines = "small_records" in name
    r = oracle.parse(data, lines=lines)
    assert r.flags == 0
    if not lines:
        assert r.n_structural == S
        assert r.n_opens == opens
