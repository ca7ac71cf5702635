"""Generates tests/golden/plan_golden.json: the JSON-Lines chunk plans of the
reference's own loaders (cujson/load_file.cu: loadJSONLines_chunkCount,
loadJSONLines_chunkSizeBytes, loadJSONLines_chunkSizeMegaBytes), run here on
the CPU (oracle/_ref/ref_loader, built by oracle/build_ref.py), for the inputs
of tests/golden/plan_cases.py.  tests/test_plan_golden.py checks the host and
device planners against them.

usage: python tests/golden/make_plan_golden.py   (needs the reference tree)
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from oracle import build_ref  # noqa: E402
from tests.golden import plan_cases  # noqa: E402

OUT = HERE / "plan_golden.json"


def sizes_digest(sizes) -> str:
    return hashlib.sha256(b"".join(int(x).to_bytes(8, "little") for x in sizes)).hexdigest()


def ref_plan(exe: Path, path: Path, mode: str, n: int):
    """(chunkCount, offsets, sizes) as the reference's loader returns them."""
    r = subprocess.run([str(exe), str(path), mode, str(n)], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"reference loader failed ({mode} {n}): rc {r.returncode} {r.stderr[-500:]}")
    rows = r.stdout.split("\n")
    count = int(rows[0])
    pairs = [tuple(int(x) for x in ln.split()) for ln in rows[1:] if ln.strip()]
    return count, [p[0] for p in pairs], [p[1] for p in pairs]


def ref_chunk_sizes(data, chunk_count: int):
    """Chunk sizes of loadJSONLines_chunkCount for in-memory bytes (used by the
    other golden generators for their JSON-Lines cases)."""
    exe = build_ref.build()["ref_loader"]
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "in.jsonl"
        p.write_bytes(bytes(data))
        count, offs, sizes = ref_plan(exe, p, "count", chunk_count)
    assert count == chunk_count == len(sizes)
    return sizes


def main():
    exes = build_ref.build()
    if "ref_loader" not in exes:
        sys.exit("reference tree not found; nothing generated")
    exe = exes["ref_loader"]
    cases = []
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "in.jsonl"
        for name, kind, args in plan_cases.CASES:
            data = plan_cases.build(kind, args)
            path.write_bytes(data.tobytes())
            plans = []
            modes = ([("count", n) for n in plan_cases.COUNTS] + [("bytes", n) for n in plan_cases.BYTE_LIMITS]
                     + [("megabytes", n) for n in plan_cases.MEGABYTES])
            for mode, n in modes:
                count, offs, sizes = ref_plan(exe, path, mode, n)
                # the loaders' chunks are contiguous: each starts where the one before ends
                pos = 0
                for o, s in zip(offs, sizes):
                    assert o == pos, (name, mode, n)
                    pos += s
                assert len(sizes) == (count if mode == "count" else len(sizes))
                plan = {"mode": mode, "n": n, "chunk_count": count, "n_chunks": len(sizes)}
                if len(sizes) <= 64:
                    plan["sizes"] = sizes
                else:   # long plans as a digest of the sizes (little-endian uint64)
                    plan["sha_sizes"] = sizes_digest(sizes)
                plans.append(plan)
            cases.append({"name": name, "kind": kind, "args": args, "size": int(data.size),
                          "sha256": hashlib.sha256(data.tobytes()).hexdigest(), "plans": plans})
            print(f"{name:24s} {data.size:9d} B  {len(plans)} plans")
    OUT.write_text(json.dumps({"generator": "tests/golden/make_plan_golden.py",
                               "source": "reference cujson/load_file.cu loaders, compiled for the CPU "
                                         "(oracle/build_ref.py ref_loader)",
                               "contiguous": True, "cases": cases}, separators=(",", ":")))
    print(f"{len(cases)} cases -> {OUT} ({OUT.stat().st_size} B)")


if __name__ == "__main__":
    main()
