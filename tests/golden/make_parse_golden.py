"""Generates tests/golden/parse_golden.json: outputs of the reference's own
parse code (cujson/parse_standard_json.cu, cujson/parse_json_lines.cu and
cujson/utils.cu, run on the CPU through the emulation built by
oracle/build_ref.py) on seeded and hand-written inputs.

Each case records how to rebuild its input (the seeded generator of
cujson_gb300 with its arguments, or the bytes themselves for short hand-written
documents), the JSON-Lines chunk sizes, and what the reference returned:
status (0 a result, 1 the reference's exit() on invalid input), S, and SHA-256
digests of structural[1..S] and of pair_pos[1..S] at the opens (0 elsewhere;
the reference leaves those entries uninitialised).  tests/test_parse_golden.py
checks the oracle and the GPU against them.

usage: python tests/golden/make_parse_golden.py   (needs the reference tree)
"""
from __future__ import annotations

import base64
import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from oracle import build_ref  # noqa: E402
from tests.golden.make_plan_golden import ref_chunk_sizes  # noqa: E402
from tests import synth  # noqa: E402  (seeded inputs)

OUT = HERE / "parse_golden.json"

HAND = [
    b'{"a":1,"b":[1,2,{"c":"x"}],"d":{"e":null}}',
    b'[{"k":"v"},{"k":"w","n":[1,[2,3]]}, 5, "s", true]',
    b'{"s":"a\\"b","t":"c\\\\","u":"{[,:]}","v":[{"w":{"x":[]}}]}',
    b'["\\\\\\"",1,"\\\\\\\\",{"\\"":"\\\\"}]',
    b'{"name":"caf\xc3\xa9","arr":["\xe2\x82\xac","\xf0\x9f\x98\x80",-1.5e+3,false]}',
    b'  [ 1 , { "a" : [ ] } ]  ',
    b'"just a string with { and ["',
    b"12345",
    b"[]",
    b"{}",
    b'[[[[[[[[[[{"deep":[[[[[]]]]]}]]]]]]]]]]',
]

# (name, kind, generator arguments); sizes stay small enough for the emulation
SYNTH = [
    ("doc_1k", "document", dict(seed=0x601D0001, size=1000, max_depth=6)),
    ("doc_4095", "document", dict(seed=0x601D0002, size=4095, max_depth=6)),
    ("doc_32k", "document", dict(seed=0x601D0003, size=32768, max_depth=10)),
    ("doc_100k", "document", dict(seed=0x601D0004, size=100003, max_depth=20)),
    ("doc_300k", "document", dict(seed=0x601D0005, size=300001, max_depth=6)),
    ("doc_1m", "document", dict(seed=0x601D0006, size=1 << 20, max_depth=20)),
    ("doc_huge_strings", "document", dict(seed=0x601D0007, size=600000, max_depth=20, huge_string_frac=0.05,
                                          huge_string_min=20000, huge_string_max=60000)),
    ("backslash_64k", "backslash", dict(seed=0x601D0008, body=65536)),
    ("backslash_70001", "backslash", dict(seed=0x601D0009, body=70001)),
    ("deep_200", "deep", dict(depth=200)),
    ("deep_255", "deep", dict(depth=255)),
    ("deep_300", "deep", dict(depth=300)),
    ("lines_20k", "lines", dict(seed=0x601D000A, size=20000, chunks=1)),
    ("lines_200k_c3", "lines", dict(seed=0x601D000B, size=200000, chunks=3)),
    ("lines_1m_c4", "lines", dict(seed=0x601D000C, size=1 << 20, chunks=4)),
]

# seeded documents with one planted error (the reference's verdict is recorded
# as observed; its UTF-8 predicate misses some classes)
CORRUPT = [
    ("bad_overlong2", dict(seed=0x601D0010, size=5000, max_depth=6), synth.CORRUPT_OVERLONG2),
    ("bad_overlong3", dict(seed=0x601D0011, size=5000, max_depth=6), synth.CORRUPT_OVERLONG3),
    ("bad_surrogate", dict(seed=0x601D0012, size=5000, max_depth=6), synth.CORRUPT_SURROGATE),
    ("bad_unbalanced", dict(seed=0x601D0013, size=5000, max_depth=6), synth.CORRUPT_UNBALANCED),
    ("bad_mismatched", dict(seed=0x601D0014, size=5000, max_depth=6), synth.CORRUPT_MISMATCHED),
]


def make_input(kind: str, args: dict):
    """(bytes, chunk sizes or None) for a case; also used by the tests."""
    if kind == "document":
        return synth.synth_document(**args), None
    if kind == "backslash":
        return synth.synth_backslash_string(args["seed"], args["body"]), None
    if kind == "deep":
        return synth.synth_deep(args["depth"]), None
    if kind == "lines":
        # the chunk sizes are the reference loader's, stored with the case
        d, _ = synth.synth_lines(args["seed"], args["size"])
        return d, None
    raise ValueError(kind)


def digests(pos: np.ndarray, pair: np.ndarray):
    return (hashlib.sha256(pos.astype("<i4").tobytes()).hexdigest(),
            hashlib.sha256(pair.astype("<i4").tobytes()).hexdigest())


def run_ref(exe: Path, data: np.ndarray, chunks, tmp: Path):
    inp, out = tmp / "in.json", tmp / "out.bin"
    inp.write_bytes(data.tobytes())
    cmd = [str(exe), str(inp), str(out)] + ([str(c) for c in chunks] if chunks else [])
    r = subprocess.run(cmd, capture_output=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"reference emulation failed: {r.stderr[-2000:]}")
    w = np.fromfile(out, dtype="<i4")
    status, S = int(w[0]), int(w[1])
    return status, S, w[2:2 + S], w[2 + S:2 + 2 * S]


def main():
    exes = build_ref.build()
    if "refemu_std" not in exes:
        sys.exit("reference tree not found; nothing generated")
    cases = []
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)

        def add(name, kind, source, data, chunks):
            exe = exes["refemu_lines" if chunks else "refemu_std"]
            status, S, pos, pair = run_ref(exe, data, chunks, tmp)
            sp, sq = digests(pos, pair)
            cases.append({"name": name, "kind": kind, "source": source, "chunk_sizes": chunks,
                          "ref_status": status, "S": S, "sha_positions": sp, "sha_pair_opens": sq})
            print(f"{name:22s} status {status} S {S}")

        for i, d in enumerate(HAND):
            add(f"hand_{i}", "hand", {"b64": base64.b64encode(d).decode()}, np.frombuffer(d, np.uint8), None)
        add("hand_lines", "hand", {"b64": base64.b64encode(b'{"a":1}\n[2,3]\n"x"\n{"b":{"c":[]}}\n').decode()},
            np.frombuffer(b'{"a":1}\n[2,3]\n"x"\n{"b":{"c":[]}}\n', np.uint8), [14, 19])
        for name, kind, args in SYNTH:
            data, _ = make_input(kind, args)
            chunks = ref_chunk_sizes(data, args["chunks"]) if kind == "lines" else None
            add(name, kind, {"args": args}, data, chunks)
        for name, args, k in CORRUPT:
            data, _ = make_input("document", args)
            assert synth.synth_corrupt(data, k, args["seed"])
            add(name, "corrupt", {"args": args, "corrupt": k}, data, None)
    OUT.write_text(json.dumps({"generator": "tests/golden/make_parse_golden.py",
                               "source": "reference cujson parse path, CPU emulation (oracle/build_ref.py)",
                               "cases": cases}, indent=1))
    print(f"{len(cases)} cases -> {OUT}")


if __name__ == "__main__":
    main()
