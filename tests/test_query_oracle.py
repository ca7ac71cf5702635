"""The query oracle (oracle/cj_oracle_query.c) against the reference's own
iterator: tests/golden/query_golden.json holds what cuJSONLinesIterator
answered to the real-world record loop (tests/golden/make_query_golden.py).
Also: the event generator's own count of "PushEvent" records agrees."""
import base64
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from tests.golden.make_query_golden import value_digest
from tests import synth

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "query_golden.json").read_text())


def golden_doc(oracle, name):
    d = GOLDEN["documents"][name]
    doc = np.frombuffer(base64.b64decode(d["b64"]), np.uint8).copy()
    res = oracle.parse(doc, lines=True, chunk_sizes=d["chunk_sizes"])
    assert res.valid
    # the reference answered on this exact result buffer
    assert hashlib.sha256(res.reference_layout().tobytes()).hexdigest() == d["layout_sha256"]
    return doc, res


def test_golden_shape():
    assert len(GOLDEN["queries"]) >= 40
    assert {q["doc"] for q in GOLDEN["queries"]} == set(GOLDEN["documents"])
    assert any(q["count"] > 100 for q in GOLDEN["queries"])


@pytest.mark.parametrize("q", GOLDEN["queries"],
                         ids=[f'{q["doc"]}-{q["key"] or "empty"}-{q["value"]}' for q in GOLDEN["queries"]])
def test_oracle_matches_reference_iterator(oracle, q):
    doc, res = golden_doc(oracle, q["doc"])
    key = q["key"].encode()
    if q["value"] is not None:
        n, _ = oracle.query_lines(doc, res, key, q["value"].encode())
        assert n == q["count"]
    else:
        n, out = oracle.query_lines(doc, res, key, None, cap=1 << 16)
        assert n == q["count"]
        assert value_digest([doc[s:s + l].tobytes() for _, s, l in out]) == q["values_sha256"]


def test_generator_push_count_matches_oracle(cj, oracle):
    doc, nrec, npush = synth.synth_events(0xC0DE5003, 1 << 20)
    res = oracle.parse(doc, lines=True)
    assert res.valid
    n, _ = oracle.query_lines(doc, res, b"type", b"PushEvent")
    assert n == npush and 0.4 * nrec < npush < 0.6 * nrec
    # every record is visited: the id key is in all of them
    assert oracle.query_lines(doc, res, b"id", None)[0] == nrec
