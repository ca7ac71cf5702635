"""Generates tests/golden/iter_golden.json: query-iterator answers of the
reference's own iterator code (cujson/query/query_iterator*.cpp, compiled by
oracle/build_ref.py) on small documents.

Each case holds the document bytes, the JSON-Lines chunk sizes, a hash of the
oracle's result buffer that the answers were taken on, a query script and the
reference's answers.  Scripts are random walks over the iterator methods with
keys drawn from the document; a script is cut before the first step that
would leave the node range [0, S], since from there the reference's loops
read outside its arrays.  tests/test_dropin.py replays every script through
the drop-in iterators (include/cujson/cujson_iter.h) and compares.

usage: python tests/golden/make_iter_golden.py   (needs the reference tree)
"""
from __future__ import annotations

import base64
import hashlib
import json
import random
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from oracle import build_ref, cj_oracle  # noqa: E402
from tests.golden.make_plan_golden import ref_chunk_sizes  # noqa: E402
from tests.dropin import build as dropin_build  # noqa: E402
from tests import synth  # noqa: E402  (seeded inputs)

OUT = HERE / "iter_golden.json"

HAND_STD = [
    b'{"a":1,"b":[1,2,{"c":"x"}],"d":{"e":null}}',
    b'[{"k":"v"},{"k":"w","n":[1,[2,3]]}, 5, "s", true]',
    b'[ { "key" : "val" , "x" : [ 1 , 2 ] } , { "key" : 3 } ]',
    b'[[1,2],[3,[4,5]],[],{}]',
    b'{"s":"a\\"b","t":"c\\\\","u":"{[,:]}","v":[{"w":{"x":[]}}]}',
    b'{"name":"caf\xc3\xa9","arr":["\xe2\x82\xac",-1.5e+3,false]}',
]
HAND_LINES = [
    b'{"type":"PushEvent","id":"1","n":[1,2]}\n{"type":"Other","id":"2"}\n'
    b'{"type":"PushEvent","id":"3","o":{"p":true}}\n{"type":"X","id":"4"}\n',
    b'[1,2,3]\n{"a":{"b":[{"c":1}]}}\n"str"\n{"a":2}',
    b'{"k": "v1", "m": 1}\n{"k": "v2", "m": [ ]}\n{"k": "v1"}\n',
]


def doc_keys(doc: bytes, lines: bool):
    keys = set()

    def walk(v):
        if isinstance(v, dict):
            for k, x in v.items():
                keys.add(k)
                walk(x)
        elif isinstance(v, list):
            for x in v:
                walk(x)

    texts = doc.split(b"\n") if lines else [doc]
    for t in texts:
        if t.strip():
            walk(json.loads(t))
    return sorted(keys)


def doc_values(doc: bytes, lines: bool):
    vals = set()
    texts = doc.split(b"\n") if lines else [doc]
    for t in texts:
        if t.strip():
            v = json.loads(t)
            if isinstance(v, dict):
                for x in v.values():
                    if isinstance(x, str):
                        vals.add(x)
    return sorted(vals)


def hexs(s: str) -> str:
    return s.encode("utf-8").hex() or "-"


def make_script(rng: random.Random, keys, values, lines: bool, steps: int, dump: bool):
    ops = ["D"] if dump else []
    for _ in range(steps):
        r = rng.random()
        if r < 0.10:
            ops.append("R")
        elif r < 0.30:
            ops.append(f"A {rng.choice([0, 0, 1, 1, 2, 3, 5, 20])}")
        elif r < 0.50:
            k = rng.choice(keys) if keys and rng.random() < 0.85 else "missing_key"
            ops.append(f"K {hexs(k)}")
        elif r < 0.58:
            k = rng.choice(keys) if keys else "x"
            ops.append(f"F {hexs(k)}")
        elif r < 0.72:
            ops.append("V")
        elif r < 0.80:
            ops.append("G")
        elif r < 0.86:
            ops.append(f"I {rng.choice([1, 1, 2, -1])}")
        elif lines and r < 0.93:
            ops.append(f"S {rng.choice([1, 1, 2])}")
        elif lines:
            k = rng.choice(keys) if keys else "x"
            v = rng.choice(values) if values and rng.random() < 0.7 else "nope"
            ops.append(f"C {hexs(k)} {hexs(v)}")
        else:
            ops.append("V")
    return ops


def layout_words(doc: bytes, lines: bool, chunk_sizes):
    res = cj_oracle.parse(np.frombuffer(doc, np.uint8), lines=lines, chunk_sizes=chunk_sizes)
    assert res.valid, doc[:80]
    buf = res.reference_layout()
    if lines:
        # per-chunk structural counts, from the chunk byte ranges
        counts, start = [], 0
        for n in chunk_sizes:
            end = start + n
            counts.append(int(((res.positions > start) & (res.positions <= end)).sum()))
            start = end
    else:
        counts = [res.n_structural]
    words = np.concatenate([np.array([res.n_structural, res.max_depth, len(counts), *counts], np.int32), buf])
    return words, hashlib.sha256(buf.tobytes()).hexdigest()


def run_driver(exe: Path, doc: bytes, words: np.ndarray, script, tmp: Path):
    (tmp / "doc.json").write_bytes(doc)
    words.astype("<i4").tofile(tmp / "layout.bin")
    (tmp / "script.txt").write_text("\n".join(script) + "\n")
    ans = tmp / "answers.txt"
    if ans.exists():
        ans.unlink()
    r = subprocess.run([str(exe), str(tmp / "doc.json"), str(tmp / "layout.bin"), str(tmp / "script.txt"),
                        str(ans)], capture_output=True, timeout=60)
    if r.returncode != 0:
        return None
    return ans.read_text().splitlines()


def compact(line: str) -> str:
    """Answer line with a long returned string replaced by a digest of it."""
    head, _, text = line.rpartition(" ")
    if len(text) > 80:
        text = "h:" + hashlib.sha256(text.encode()).hexdigest()[:20]
    return f"{head} {text}"


def truncate(answers, script, S):
    """Keep the steps before the first one that leaves node range [0, S]."""
    keep = []
    for step, a in zip(script, answers):
        node = int(a.split()[2])
        if node < 0 or node > S:
            break
        keep.append(step)
    return keep


def cases():
    rng = random.Random(0xC0DE17E5)
    out = []
    for i, d in enumerate(HAND_STD):
        out.append((f"hand_std_{i}", d, False, None))
    for i, d in enumerate(HAND_LINES):
        out.append((f"hand_lines_{i}", d, True, [len(d)]))
    for i, seed in enumerate([11, 12, 13, 14]):
        size = [1024, 2048, 4096, 6144][i]
        d = bytes(synth.synth_document(0xC0DE1000 + seed, size, max_depth=6))
        out.append((f"synth_std_{size}", d, False, None))
    for i, seed in enumerate([21, 22, 23]):
        size = [1500, 3000, 5000][i]
        d = bytes(synth.synth_lines(0xC0DE2000 + seed, size)[0])
        nchunks = [1, 2, 3][i]
        sizes = ref_chunk_sizes(np.frombuffer(d, np.uint8), nchunks)
        out.append((f"synth_lines_{size}_c{nchunks}", d, True, sizes))
    # a hand document split into several chunks
    d = HAND_LINES[0]
    out.append(("hand_lines_0_c2", d, True, ref_chunk_sizes(np.frombuffer(d, np.uint8), 2)))
    return rng, out


def main():
    ref = build_ref.build()
    if not ref:
        sys.exit("reference tree not found; nothing generated")
    ours = dropin_build.build()
    rng, items = cases()
    golden, documents = [], {}
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        for name, doc, lines, sizes in items:
            keys = doc_keys(doc, lines)
            values = doc_values(doc, lines)
            words, digest = layout_words(doc, lines, sizes)
            documents[name] = {"b64": base64.b64encode(doc).decode(), "lines": lines,
                               "chunk_sizes": sizes, "layout_sha256": digest}
            S = int(words[0])
            exe_ref = ref["iter_ref_lines" if lines else "iter_ref_std"]
            exe_ours = ours["iter_lines" if lines else "iter_std"]
            for k in range(4):
                script = make_script(rng, keys, values, lines, 60, k == 0)
                traced = run_driver(exe_ours, doc, words, script, tmp)
                script = truncate(traced, script, S)
                answers = run_driver(exe_ref, doc, words, script, tmp)
                if answers is None:
                    print(f"{name}#{k}: reference driver failed; script dropped")
                    continue
                golden.append({"doc": name, "script": script, "answers": [compact(a) for a in answers]})
    OUT.write_text(json.dumps({"generator": "tests/golden/make_iter_golden.py",
                               "source": "reference cujson/query iterators, g++",
                               "documents": documents, "cases": golden}, separators=(",", ":")))
    print(f"{len(golden)} cases -> {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
