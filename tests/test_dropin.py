"""Drop-in C++ surface: query iterators against the reference's own answers,
and the reference's example programs compiling unchanged against
include/cujson/.

The golden answers (tests/golden/iter_golden.json) were produced by the
reference's iterator code (cujson/query/query_iterator*.cpp) on the oracle's
result buffers; here the same scripts run through include/cujson/cujson_iter.h.
"""
from __future__ import annotations

import base64
import hashlib
import json
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import build_ref

from tests.dropin import build as dropin_build
from tests import synth

REPO = Path(__file__).resolve().parent.parent
GOLDEN = REPO / "tests" / "golden" / "iter_golden.json"
REFERENCE = build_ref.DEFAULT_REF


def compact(line: str) -> str:
    head, _, text = line.rpartition(" ")
    if len(text) > 80:
        text = "h:" + hashlib.sha256(text.encode()).hexdigest()[:20]
    return f"{head} {text}"


def normalise(line: str) -> str:
    # the reference throws std::length_error where a negative slice length
    # reaches std::string; the drop-in returns an empty string there
    head, _, text = line.rpartition(" ")
    return f"{head} -" if text == "exception" else line


def layout_words(oracle, doc: bytes, lines: bool, chunk_sizes):
    res = oracle.parse(np.frombuffer(doc, np.uint8), lines=lines, chunk_sizes=chunk_sizes)
    assert res.valid
    buf = res.reference_layout()
    if lines:
        counts, start = [], 0
        for n in chunk_sizes:
            end = start + n
            counts.append(int(((res.positions > start) & (res.positions <= end)).sum()))
            start = end
    else:
        counts = [res.n_structural]
    head = np.array([res.n_structural, res.max_depth, len(counts), *counts], np.int32)
    return np.concatenate([head, buf]), hashlib.sha256(buf.tobytes()).hexdigest()


def run_driver(exe: Path, doc: bytes, words: np.ndarray, script, tmp: Path):
    (tmp / "doc.json").write_bytes(doc)
    words.astype("<i4").tofile(tmp / "layout.bin")
    (tmp / "script.txt").write_text("\n".join(script) + "\n")
    ans = tmp / "answers.txt"
    r = subprocess.run([str(exe), str(tmp / "doc.json"), str(tmp / "layout.bin"), str(tmp / "script.txt"),
                        str(ans)], capture_output=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return ans.read_text().splitlines()


@pytest.fixture(scope="module")
def drivers():
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    return dropin_build.build()


@pytest.fixture(scope="module")
def golden():
    return json.loads(GOLDEN.read_text())


def test_golden_fixture_shape(golden):
    assert golden["cases"], "no golden cases"
    ops = {step.split()[0] for c in golden["cases"] for step in c["script"]}
    # every iterator method is exercised
    assert ops >= {"R", "A", "K", "F", "I", "V", "G", "D", "S", "C"}


def test_iterators_match_reference_answers(drivers, golden, oracle, tmp_path):
    mismatches = []
    for name, d in golden["documents"].items():
        doc = base64.b64decode(d["b64"])
        words, digest = layout_words(oracle, doc, d["lines"], d["chunk_sizes"])
        # the answers were taken on this exact result buffer
        assert digest == d["layout_sha256"], name
        exe = drivers["iter_lines" if d["lines"] else "iter_std"]
        for case in (c for c in golden["cases"] if c["doc"] == name):
            got = [compact(a) for a in run_driver(exe, doc, words, case["script"], tmp_path)]
            want = [normalise(a) for a in case["answers"]]
            assert len(got) == len(want)
            for i, (g, w) in enumerate(zip(got, want)):
                if g != w:
                    mismatches.append((name, i, case["script"][i], w, g))
                    break
    assert not mismatches, mismatches[:5]


def test_real_world_query_pattern(drivers, oracle, tmp_path):
    """The PushEvent count loop of the reference's real-world example: reset,
    gotoArrayIndex(0), then per record checkKeyValue / gotoKey / gotoNextSibling."""
    recs, want = [], 0
    rng = np.random.default_rng(7)
    for i in range(200):
        t = "PushEvent" if rng.random() < 0.3 else "WatchEvent"
        want += t == "PushEvent"
        recs.append(f'{{"id":"{i}","type":"{t}","payload":{{"size":{i % 5}}}}}')
    doc = ("\n".join(recs) + "\n").encode()
    words, _ = layout_words(oracle, doc, True, [len(doc)])
    script = ["R", "A 0"]
    for _ in range(200):
        script += [f"C {b'type'.hex()} {b'PushEvent'.hex()}", "S 1"]
    ans = run_driver(drivers["iter_lines"], doc, words, script, tmp_path)
    hits = sum(1 for s, a in zip(script, ans) if s.startswith("C") and a.split()[1] == "1")
    assert hits == want


EXAMPLES = ["main.cu", "main_jsonlines.cu", "main_jsonlines_chunksize.cu", "main_jsonlines_chunksize_MB.cu"]


@pytest.mark.parametrize("example", EXAMPLES)
def test_reference_examples_compile_unchanged(example, cj, tmp_path):
    """The reference's example programs compile and link, unmodified, against
    include/cujson/ and libcujson_gb300 (the reference tree is only read)."""
    src = REFERENCE / example
    if not src.exists():
        pytest.skip("reference examples not present")
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not available")
    work = tmp_path / "ex"
    work.mkdir()
    shutil.copy(src, work / example)
    libdir = Path(cj.lib()._name).parent
    cmd = ["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{REPO / 'include'}",
           str(work / example), "-o", str(work / "a.out"), f"-L{libdir}", "-lcujson_gb300",
           f"-Xlinker", f"-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]


def test_example_program_builds(cj):
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not available")
    exe = dropin_build.build_example(Path(cj.lib()._name).parent)
    assert exe.exists()


def _read_layout(path: Path):
    w = np.fromfile(path, dtype="<i4")
    S, depth, n = int(w[0]), int(w[1]), int(w[2])
    return S, depth, w[3:3 + n], w[3 + n:]


@pytest.mark.gpu
@pytest.mark.parametrize("mode,arg", [("std", None), ("lines", 1), ("lines", 3), ("lines_mb", 1)])
def test_example_program_on_gpu(cj, oracle, tmp_path, mode, arg):
    """A user program over the drop-in headers: loadJSON / loadJSONLines_*,
    parse_*, iterator, freeJson -- its result buffer equals the oracle's."""
    exe = dropin_build.build_example(Path(cj.lib()._name).parent)
    f = tmp_path / "doc.json"
    if mode == "std":
        doc = synth.synth_document(0xD0C0001, 3 << 20, max_depth=12)
        f.write_bytes(doc.tobytes())
        args = [str(exe), mode, str(f), str(tmp_path / "out.bin")]
        ref = oracle.parse(doc)
    else:
        doc, _ = synth.synth_lines(0xD0C0002, 3 << 20)
        f.write_bytes(doc.tobytes())
        args = [str(exe), mode, str(f), str(arg), str(tmp_path / "out.bin")]
        sizes = (cj.plan_lines_count(doc, arg) if mode == "lines"
                 else cj.plan_lines_bytes(doc, arg << 20))
        ref = oracle.parse(doc, lines=True, chunk_sizes=sizes)
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("first: ")
    S, depth, _, buf = _read_layout(tmp_path / "out.bin")
    assert S == ref.n_structural and depth == ref.max_depth
    np.testing.assert_array_equal(buf, ref.reference_layout())
