"""JSON-Lines chunk planning pinned to the reference's own loaders.

tests/golden/plan_golden.json holds the chunk plans that the reference's
loadJSONLines_chunkCount / _chunkSizeBytes / _chunkSizeMegaBytes
(cujson/load_file.cu:38, :109, :182) returned, compiled for the CPU and run on
the inputs of tests/golden/plan_cases.py (make_plan_golden.py).  The cases
cover a last line without a newline, more chunks than lines, a first line
longer than the byte limit (an empty first chunk, load_file.cu:161-166), empty
files and lines, CRLF, and newlines on the device planner's 64 KiB block edges.

The host planners (cj_plan_lines_count, cj_plan_lines_bytes) are checked here
on the CPU, the device planner (cj_plan_lines_count_device) on the GPU, all
against the same goldens.
"""
import hashlib
import json
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from tests.golden import plan_cases
from tests.golden.make_plan_golden import sizes_digest

GOLDEN = Path(__file__).resolve().parent / "golden" / "plan_golden.json"
DATA = json.loads(GOLDEN.read_text())
CASES = DATA["cases"]
REF_LOADER = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "ref_loader"


def case_bytes(c):
    data = plan_cases.build(c["kind"], c["args"])
    assert data.size == c["size"] and hashlib.sha256(data.tobytes()).hexdigest() == c["sha256"], c["name"]
    return data


def assert_plan(got, plan, what):
    assert len(got) == plan["n_chunks"], what
    if "sizes" in plan:
        assert list(got) == plan["sizes"], what
    else:
        assert sizes_digest(got) == plan["sha_sizes"], what


def test_golden_covers_the_edge_cases():
    names = {c["name"] for c in CASES}
    assert len(CASES) >= 10
    assert {"one_line_no_newline", "first_line_over_limit", "empty_file", "only_newlines"} <= names
    # the reference's empty first chunk for a first line over the byte limit
    c = next(c for c in CASES if c["name"] == "first_line_over_limit")
    p = next(p for p in c["plans"] if p["mode"] == "bytes" and p["n"] == 4096)
    assert p["sizes"][0] == 0
    # more chunks than lines: trailing empty chunks
    c = next(c for c in CASES if c["name"] == "empty_lines")
    p = next(p for p in c["plans"] if p["mode"] == "count" and p["n"] == 64)
    assert p["n_chunks"] == 64 and p["sizes"][-1] == 0


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_host_planners_match_reference_loaders(cj, c):
    data = case_bytes(c)
    for plan in c["plans"]:
        what = (c["name"], plan["mode"], plan["n"])
        if plan["mode"] == "count":
            got = cj.plan_lines_count(data, plan["n"])
            assert plan["chunk_count"] == plan["n"], what
        else:
            limit = plan["n"] << 20 if plan["mode"] == "megabytes" else plan["n"]
            got = cj.plan_lines_bytes(data, limit)
            assert plan["chunk_count"] == len(got), what
        assert_plan(got, plan, what)
        assert sum(got) == data.size, what


def _ref_loader_plan(path, mode, n):
    r = subprocess.run([str(REF_LOADER), str(path), mode, str(n)], capture_output=True, text=True, check=True)
    rows = [ln.split() for ln in r.stdout.strip().split("\n")[1:] if ln.strip()]
    return [int(s) for _, s in rows]


@pytest.mark.skipif(not REF_LOADER.exists(), reason="reference loader not built (reference tree absent)")
def test_host_planners_match_reference_loaders_random():
    """Beyond the goldens, where the reference's loader is built: random
    buffers of lines, blank lines, long lines and an open last line."""
    import cujson_gb300 as cj
    rng = np.random.default_rng(0x601D7100)
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "in.jsonl"
        for _ in range(40):
            n = int(rng.integers(0, 20000))
            buf = np.where(rng.random(n) < rng.choice([0.001, 0.02, 0.3]), ord("\n"), ord("z")).astype(np.uint8)
            path.write_bytes(buf.tobytes())
            for k in (1, 2, 5, int(rng.integers(1, 300))):
                assert cj.plan_lines_count(buf, k) == _ref_loader_plan(path, "count", k)
            for lim in (0, 1, int(rng.integers(1, 4000)), 100000):
                assert cj.plan_lines_bytes(buf, lim) == _ref_loader_plan(path, "bytes", lim)


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_device_planner_matches_reference_loaders(ctx, c):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    data = case_bytes(c)
    d = torch.from_numpy(data.copy()).to("cuda") if data.size else None
    torch.cuda.synchronize()
    ptr = d.data_ptr() if d is not None else 0
    for plan in c["plans"]:
        what = (c["name"], plan["mode"], plan["n"])
        if plan["mode"] == "count":
            got = ctx.plan_lines_count_device(ptr, int(data.size), plan["n"])
        else:
            limit = plan["n"] << 20 if plan["mode"] == "megabytes" else plan["n"]
            got = ctx.plan_lines_bytes_device(ptr, int(data.size), limit)
            assert plan["chunk_count"] == len(got), what
        assert_plan(got, plan, what)
