"""Parse parity against golden outputs of the reference's own parse code.

tests/golden/parse_golden.json holds, per input, what the reference's
parse_standard_json / parse_json_lines returned when its CUDA sources were run
on the CPU (oracle/build_ref.py emulation; tests/golden/make_parse_golden.py):
its status and digests of structural[1..S] and of pair_pos at the opens.  The
oracle (CPU) and the GPU path must reproduce them bit for bit, except for the
documented divergences below, where the reference is wrong by design of this
project (strict UTF-8, int32 depth) and the expected verdict is stated.
"""
import base64
import json
from pathlib import Path

import numpy as np
import pytest

from tests.golden.make_parse_golden import digests, make_input
from tests import synth

GOLDEN = Path(__file__).resolve().parent / "golden" / "parse_golden.json"
CASES = json.loads(GOLDEN.read_text())["cases"]

# case -> (why the reference differs, the verdict expected here)
DIVERGENCES = {
    "bad_overlong2": ("the reference's UTF-8 predicate accepts the overlong C0 80", "utf8"),
    "bad_overlong3": ("the reference's UTF-8 predicate accepts the overlong E0 80 80", "utf8"),
    "bad_surrogate": ("the reference's UTF-8 predicate accepts the surrogate ED A0 80", "utf8"),
    "deep_300": ("the reference's uint8 depth wraps past 256 and it exits", "valid"),
}


def case_input(c):
    if c["kind"] == "hand":
        return np.frombuffer(base64.b64decode(c["source"]["b64"]), np.uint8).copy(), c["chunk_sizes"]
    if c["kind"] == "corrupt":
        import cujson_gb300 as cj
        data, _ = make_input("document", c["source"]["args"])
        assert synth.synth_corrupt(data, c["source"]["corrupt"], c["source"]["args"]["seed"])
        return data, None
    data, chunks = make_input(c["kind"], c["source"]["args"])
    return data, c["chunk_sizes"]


def check(c, valid, positions, pair_row, utf8_flag):
    name = c["name"]
    if name in DIVERGENCES:
        _, want = DIVERGENCES[name]
        if want == "utf8":
            assert not valid and utf8_flag, name
        else:
            assert valid, name
        return
    if c["ref_status"] != 0:
        assert not valid, name
        return
    assert valid, name
    assert len(positions) == c["S"], name
    sp, sq = digests(np.asarray(positions), np.asarray(pair_row))
    assert sp == c["sha_positions"], name
    assert sq == c["sha_pair_opens"], name


def test_golden_cases_present():
    names = {c["name"] for c in CASES}
    assert len(CASES) >= 30 and set(DIVERGENCES) <= names
    # the reference answered most cases with a result, and rejected the bad brackets
    assert sum(c["ref_status"] == 0 for c in CASES) >= 25


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference(oracle, c):
    data, chunks = case_input(c)
    r = oracle.parse(data, lines=chunks is not None, chunk_sizes=chunks)
    check(c, r.flags == 0, r.positions, r.pair_row, bool(r.flags & oracle.ERR_UTF8))


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_gpu_matches_reference(cj, ctx, c):
    data, chunks = case_input(c)
    st, res = ctx.try_parse(data, lines=chunks is not None, chunk_sizes=chunks)
    if st == cj.OK:
        check(c, True, res.positions, res.pair_row, False)
    else:
        check(c, False, [], [], st == cj.ERR_INVALID_UTF8)
