"""Generates tests/golden/query_golden.json: answers of the reference's own
iterator code (cujson/query/query_iterator.cpp, compiled by oracle/build_ref.py
into iter_ref_lines) to the real-world record loop of
real_world_use_case/main.cu:70-86 -- gotoArrayIndex(0), then per record
checkKeyValue(key, value) (or findKey / gotoKey / getValue) and
gotoNextSibling(1) -- on seeded event-log files and hand-written edge cases.

Per query it stores the number of records answered true (checkKeyValue) or
that have the key, and for key-only queries a digest of the values in visiting
order.  tests/test_query_oracle.py checks the oracle's restatement
(oracle/cj_oracle_query.c) against these; the GPU tests check the device query
engine against both.

usage: python tests/golden/make_query_golden.py   (needs the reference tree)
"""
from __future__ import annotations

import base64
import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from oracle import build_ref, cj_oracle  # noqa: E402
from tests.golden.make_plan_golden import ref_chunk_sizes  # noqa: E402
from tests.golden.make_iter_golden import layout_words, run_driver  # noqa: E402
from tests import synth  # noqa: E402  (seeded inputs)

OUT = HERE / "query_golden.json"

HAND = {
    "hand_mix": (
        b'{"id":1,"type":"PushEvent"}\n'
        b'{"type" : "WatchEvent","a":{"type":"PushEvent"}}\n'
        b'{"a":{"type":"PushEvent"}, "type": "PushEvent"},{"type":"PushEvent"}\n'
        b'\n'
        b'{"b":2}\n'
        b'[{"type":"PushEvent"}]\n'
        b'{"type":""}\n'
        b'{"type":"Push\\"Event"}\n'
        b'{"type":{"x":1}}\n'
        b'{"type":[1,[2]],"type":"PushEvent"}\n'
        b'{"type":123}\n'
        b'{  "type"  :   "PushEvent"  }\n'
        b'{"type":" PushEvent "}\n'
        b'{"x":[{"type":"PushEvent"}],"type":"PushEvent","y":{}}\n'
        b'"str"\n'
        b'12\n'
        b'{"type":"PushEvent"}'
    ),
    # records and values that span lines: the iterator jumps records whole,
    # so a '{' after a newline inside a record is not a record
    "hand_multiline": (
        b'{"type":\n"PushEvent","a":1}\n'
        b'{"x":{"type":"PushEvent"},\n"type":"PushEvent"}\n'
        b'{"a":[\n{"type":"PushEvent"}\n],"type":"WatchEvent"}\n'
        b'[{"type":"PushEvent"},\n{"type":"X"}]\n'
        b'{"type" :\n "PushEvent" }\n'
        b'{"type":"PushEvent"}\n'
        b'{\n"id":7,\n"type":"PushEvent"\n}\n'
    ),
    "hand_keys": (
        b'{"":1,"type":null}\n'
        b'{"t":"PushEvent","tt":{"":"x"}}\n'
        b'{"k":true,"":"empty-key"}\n'
        b'{"type":"caf\xc3\xa9","n":-1.5e+3}\n'
    ),
}

QUERIES = [("type", "PushEvent"), ("type", "WatchEvent"), ("type", "PushEventX"), ("type", ""),
           ("type", None), ("payload", None), ("id", None), ("public", None), ("org", None),
           ("missing", None), ("", None), ("", "1")]


def cases():
    out = []
    for name, d in HAND.items():
        out.append((name, d, [len(d)]))
    d = bytes(synth.synth_events(0xC0DE5001, 256 << 10)[0])
    out.append(("events_256k", d, [len(d)]))
    d = bytes(synth.synth_events(0xC0DE5002, 192 << 10)[0])
    out.append(("events_192k_c3", d, ref_chunk_sizes(np.frombuffer(d, np.uint8), 3)))
    return out


def value_digest(values) -> str:
    h = hashlib.sha256()
    for v in values:
        h.update(len(v).to_bytes(4, "little"))
        h.update(v)
    return h.hexdigest()


def reference_answer(exe, doc, words, key: str, value, tmp):
    kh = key.encode().hex() or "-"
    res = cj_oracle.parse(np.frombuffer(doc, np.uint8), lines=True)
    chars = np.frombuffer(doc, np.uint8)[res.positions - 1]
    bound = int(np.count_nonzero((chars == ord(",")) | (chars == ord("\n")))) + 2
    script = ["R", "A 0"]
    if value is not None:
        vh = value.encode().hex() or "-"
        script += [f"C {kh} {vh}", "S 1"] * bound
    else:
        script += [f"F {kh}", f"K {kh}", "V", "S 1"] * bound
    ans = run_driver(exe, doc, words, script, tmp)
    assert ans is not None and len(ans) == len(script)
    count, values = 0, []
    i = 2
    while i < len(script):
        if value is not None:
            count += ans[i].split()[1] == "1"
            step = 2
        else:
            if ans[i].split()[1] != "0":
                text = ans[i + 2].split()[-1]
                values.append(b"" if text == "-" else bytes.fromhex(text))
                count += 1
            step = 4
        if ans[i + step - 1].split()[1] == "0":     # gotoNextSibling failed: past the last record
            break
        i += step
    return count, values


def main():
    ref = build_ref.build()
    if not ref:
        sys.exit("reference tree not found; nothing generated")
    exe = ref["iter_ref_lines"]
    documents, golden = {}, []
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        for name, doc, sizes in cases():
            words, digest = layout_words(doc, True, sizes)
            documents[name] = {"b64": base64.b64encode(doc).decode(), "chunk_sizes": sizes,
                               "layout_sha256": digest}
            for key, value in QUERIES:
                count, values = reference_answer(exe, doc, words, key, value, tmp)
                rec = {"doc": name, "key": key, "value": value, "count": count}
                if value is None:
                    rec["values_sha256"] = value_digest(values)
                golden.append(rec)
                print(name, repr(key), repr(value), count)
    OUT.write_text(json.dumps({"documents": documents, "queries": golden}, indent=1) + "\n")
    print(f"wrote {OUT}: {len(golden)} queries")


if __name__ == "__main__":
    main()
