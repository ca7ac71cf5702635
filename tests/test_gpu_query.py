"""The device query engine (cj_query_count / cj_query_values) against the
reference's own iterator answers (tests/golden/query_golden.json) and the
oracle's restatement of the reference's record loop, bit for bit: counts,
record offsets, value offsets and lengths.  At full size on a 2 GB event-log
file the oracle and the generator's own count are the checks."""
import base64
import json
from pathlib import Path

import numpy as np
import pytest

from tests.golden.make_query_golden import value_digest
from tests import synth

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "query_golden.json").read_text())


def staged(ctx, doc, sizes):
    offs = np.concatenate([[0], np.cumsum(sizes)])
    res = ctx.parse_json_lines([doc[offs[i]:offs[i + 1]] for i in range(len(sizes))])
    return res


@pytest.mark.parametrize("name", sorted(GOLDEN["documents"]))
def test_golden_queries(cj, oracle, ctx, name):
    d = GOLDEN["documents"][name]
    doc = np.frombuffer(base64.b64decode(d["b64"]), np.uint8).copy()
    staged(ctx, doc, d["chunk_sizes"])
    ref = oracle.parse(doc, lines=True, chunk_sizes=d["chunk_sizes"])
    for q in (q for q in GOLDEN["queries"] if q["doc"] == name):
        key = q["key"].encode()
        if q["value"] is not None:
            assert ctx.query_count(key, q["value"].encode()) == q["count"], q
        else:
            got = ctx.query_values(key)
            assert got.shape[0] == q["count"], q
            assert value_digest([doc[s:s + l].tobytes() for _, s, l in got]) == q["values_sha256"], q
            n, want = oracle.query_lines(doc, ref, key, None, cap=max(1, q["count"]))
            np.testing.assert_array_equal(got, want)


def test_events_full_size(cj, oracle, ctx):
    """2 GB of event-log records (the JSON-Lines size limit)."""
    doc, nrec, npush = synth.synth_events(0xC0DE5004, cj.MAX_INPUT_BYTES)
    sizes = cj.plan_lines_count(doc, 4)
    res = staged(ctx, doc, sizes)
    ref = oracle.parse(doc, lines=True, chunk_sizes=sizes)
    assert res.n_structural == ref.n_structural
    assert ctx.query_count(b"type", b"PushEvent") == npush
    assert ctx.query_count(b"type", b"WatchEvent") == oracle.query_lines(doc, ref, b"type", b"WatchEvent")[0]
    got = ctx.query_values(b"type")
    n, want = oracle.query_lines(doc, ref, b"type", None, cap=nrec)
    assert got.shape[0] == n
    np.testing.assert_array_equal(got, want)
    assert ctx.query_values(b"id").shape[0] == nrec


def test_random_keys_config3_shape(cj, oracle, ctx):
    """The 2 GB JSON-Lines workload's own records (random keys): the first
    record's first key, extracted everywhere it occurs at top level."""
    doc, _ = synth.synth_lines(synth.CONFIG_SEED_BASE + 3, 256 << 20)
    sizes = cj.plan_lines_count(doc, 2)
    staged(ctx, doc, sizes)
    ref = oracle.parse(doc, lines=True, chunk_sizes=sizes)
    head = doc[:64].tobytes()
    key = head[2:head.index(b'"', 2)]
    got = ctx.query_values(key)
    n, want = oracle.query_lines(doc, ref, key, None, cap=1 << 16)
    assert n >= 1 and got.shape[0] == n
    np.testing.assert_array_equal(got, want[:n])


def test_capacity_multiline_and_refusals(cj, ctx):
    doc = np.frombuffer(b'{"type":"A"}\n{"type":"B"}\n{"type":"A"}\n', np.uint8)
    ctx.parse_json_lines([doc])
    assert ctx.query_count(b"type", b"A") == 2
    with pytest.raises(cj.CujsonError) as e:
        ctx.query_values(b"type", cap=2)
    assert e.value.status == cj.ERR_CAPACITY
    # records that span lines are jumped whole, as the iterator's walk does
    ml = np.frombuffer(b'{"type":"A",\n"b":{"type":"A"}}\n{"c":[\n{"type":"A"}]}\n{"type":"A"}\n', np.uint8)
    ctx.parse_json_lines([ml])
    assert ctx.query_count(b"type", b"A") == 2
    # standard JSON and batches are not JSON-Lines results
    ctx.parse_standard_json(np.frombuffer(b'[{"type":"A"}]', np.uint8))
    with pytest.raises(cj.CujsonError) as e:
        ctx.query_count(b"type", b"A")
    assert e.value.status == cj.ERR_NOT_STAGED
    # keys and values are at most 256 bytes
    ctx.parse_json_lines([doc])
    with pytest.raises(cj.CujsonError) as e:
        ctx.query_count(b"k" * 257, b"A")
    assert e.value.status == cj.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("seed", [11, 12, 13, 14, 15])
def test_random_documents_and_keys(cj, oracle, ctx, seed):
    """Random-key JSON Lines (the config-3 generator, several chunkings) and
    event logs: keys drawn from the documents' records -- the records' own
    top-level keys and nested keys -- counted and extracted on the device and
    by the oracle, bit for bit."""
    rng = np.random.default_rng(seed)
    if seed % 2:
        doc, _ = synth.synth_lines(seed, 3 << 20, max_depth=4)
    else:
        doc, _, _ = synth.synth_events(seed, 3 << 20)
    n_chunks = int(rng.integers(1, 5))
    sizes = cj.plan_lines_count(doc, n_chunks)
    staged(ctx, doc, sizes)
    ref = oracle.parse(doc, lines=True, chunk_sizes=sizes)
    text = doc.tobytes()
    # candidate keys: every quoted token followed by ':' in a few sampled lines
    keys = set()
    starts = np.flatnonzero(doc == ord("\n")) + 1
    for st in rng.choice(starts[:-1], size=min(8, starts.size - 1), replace=False):
        line = text[st:text.index(b"\n", st)]
        i = 0
        while len(keys) < 24:
            a = line.find(b'"', i)
            if a < 0:
                break
            b = line.find(b'"', a + 1)
            if b < 0:
                break
            if line[b + 1:b + 2] == b":" and b - a - 1 <= 64 and b"\\" not in line[a + 1:b]:
                keys.add(line[a + 1:b])
            i = b + 1
    assert keys
    for key in sorted(keys):
        n, want = oracle.query_lines(doc, ref, key, None, cap=1 << 18)
        got = ctx.query_values(key)
        assert got.shape[0] == n, key
        np.testing.assert_array_equal(got, want[:n], err_msg=str(key))
        if n:
            # count the records whose value equals the first match's value
            s, l = int(want[0, 1]), int(want[0, 2])
            value = text[s:s + l][:256]
            if len(text[s:s + l]) <= 256:
                assert ctx.query_count(key, value) == oracle.query_lines(doc, ref, key, value)[0], key
