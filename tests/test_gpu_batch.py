"""Batches of independent documents (one run for many documents) against the
oracle and against single-document parses: per-document arrays bit-exact,
per-document verdicts, graph replays and autotuned launch shapes giving the
same results."""
import numpy as np
import pytest
from tests import synth

pytestmark = pytest.mark.gpu


def check_batch(cj, oracle, docs, results):
    assert len(results) == len(docs)
    for i, (d, (st, res)) in enumerate(zip(docs, results)):
        ref = oracle.parse(d)
        if ref.flags:
            want = cj.ERR_INVALID_UTF8 if ref.flags & oracle.ERR_UTF8 else cj.ERR_INVALID_BRACKETS
            assert st == want, (i, st, ref.flags)
        else:
            assert st == cj.OK, (i, st)
            assert res.n_structural == ref.n_structural, i
            np.testing.assert_array_equal(res.buffer, ref.reference_layout(), err_msg=f"doc {i}")
            assert res.max_depth == ref.max_depth, i


def mixed_docs(cj, seed=7):
    docs = [np.frombuffer(b, np.uint8).copy() for b in (
        b"1", b"[]", b'{"a":"b\\"c,d"}', b"[[[", b"[1,[2]]", b"]]", b"{}", b"[{]}", b"[]",
        b'"\\\\"', b"   ", b'{"k":[{},[]],"x":{}}', b"\xc0\x80", b'["\xed\xa0\x80"]', b"[\"\xe2\x82\xac\"]")]
    for k, n in enumerate([1023, 1024, 1025, 4095, 65536, 114687, 114688, 114689, 131072, 300001, 1 << 20]):
        docs.append(synth.synth_document(seed * 100 + k, n, max_depth=10))
    bad = synth.synth_document(seed * 100 + 50, 200000)
    assert synth.synth_corrupt(bad, synth.CORRUPT_SURROGATE, 3)
    docs.append(bad)
    bad2 = synth.synth_document(seed * 100 + 51, 150000)
    assert synth.synth_corrupt(bad2, synth.CORRUPT_MISMATCHED, 3)
    docs.append(bad2)
    docs.append(synth.synth_deep(100000))
    docs.append(synth.synth_backslash_string(seed, 300000))
    return docs


def test_batch_per_document_pointers(cj, oracle, ctx):
    docs = mixed_docs(cj)
    ctx.stage_batch(docs)
    ctx.run()
    check_batch(cj, oracle, docs, ctx.batch_results())


def test_batch_packed_and_graph(cj, oracle, ctx):
    docs = mixed_docs(cj, seed=8)
    packed = np.concatenate(docs)
    ctx.stage_batch_packed(packed, [d.size for d in docs])
    ctx.run_graph()
    first = ctx.batch_layout()[0].copy()
    check_batch(cj, oracle, docs, ctx.batch_results())
    ctx.run_graph()          # replay
    np.testing.assert_array_equal(ctx.batch_layout()[0], first)
    ctx.run()                # the same staged batch without the graph
    np.testing.assert_array_equal(ctx.batch_layout()[0], first)


def test_batch_same_alone_and_in_the_mix(cj, ctx):
    docs = mixed_docs(cj, seed=9)
    ctx.stage_batch(docs)
    ctx.run()
    mixed = ctx.batch_results()
    for i, d in enumerate(docs):
        st, res = ctx.try_parse(d)
        assert st == mixed[i][0], i
        if st == cj.OK:
            np.testing.assert_array_equal(res.buffer, mixed[i][1].buffer)


def test_batch_generated(cj, oracle, ctx):
    packed, sizes, kinds = synth.batch_input(0xC0DE1004, 300, 96 << 20)
    ctx.stage_batch_packed(packed, sizes)
    ctx.run_graph()
    res = ctx.batch_results()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    docs = [packed[offs[i]:offs[i + 1]] for i in range(sizes.size)]
    check_batch(cj, oracle, docs, res)
    assert sum(1 for st, _ in res if st != cj.OK) == int((kinds > 0).sum())


def test_autotune_keeps_results(cj, oracle, ctx):
    packed, sizes, _ = synth.batch_input(0xC0DE2004, 64, 16 << 20)
    ctx.stage_batch_packed(packed, sizes)
    ctx.run_graph()
    want = ctx.batch_layout()[0].copy()
    best, tried = ctx.autotune(reps=2)
    assert len(tried) >= 6 and best.ms > 0
    assert min(t.ms for t in tried) == pytest.approx(best.ms)
    ctx.run_graph()
    np.testing.assert_array_equal(ctx.batch_layout()[0], want)
    assert {t.prefetch_steps for t in tried} == {2, 4, 8} and {t.region_kib for t in tried} == {4, 8, 16}
    # the winner kept in a file keyed by GPU name, and applied again
    import tempfile, os
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "tuning.jsonl")
        with open(path, "w") as f:
            f.write('{"gpu": "another GPU", "region_kib": 4}\n')
        ctx.save_tuning(path)
        ctx.set_tuning()
        ctx.load_tuning(path)
        got = ctx.get_tuning()
        for k in ("region_kib", "scan_blocks_per_sm", "pair_blocks", "pair_threads", "prefetch_steps"):
            assert getattr(got, k) == getattr(best, k), k
        lines = open(path).read().splitlines()
        assert len(lines) == 2 and lines[0].startswith('{"gpu": "another GPU"')
        with open(path, "w") as f:
            f.write('{"gpu": "another GPU", "region_kib": 4}\n')
        with pytest.raises(cj.CujsonError):
            ctx.load_tuning(path)
    ctx.run_graph()
    np.testing.assert_array_equal(ctx.batch_layout()[0], want)
    ctx.set_tuning()   # back to defaults for the other tests


def test_single_document_after_batch(cj, oracle, ctx):
    d = synth.synth_document(1234, 500000)
    st, res = ctx.try_parse(d)
    assert st == cj.OK
    np.testing.assert_array_equal(res.buffer, oracle.parse(d).reference_layout())
    ctx.stage_standard(d)
    ctx.run_graph()
    np.testing.assert_array_equal(ctx.staged_result().buffer, res.buffer)


def padded_copy(cj, docs_or_packed, sizes, pinned=True):
    """The documents laid out at batch_padded_offsets (a pinned buffer)."""
    off, total = cj.batch_padded_offsets(sizes)
    buf = cj.PinnedBuffer(max(total, 1)) if pinned else None
    arr = buf.array if pinned else np.zeros(max(total, 1), np.uint8)
    src = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    for i in range(len(sizes)):
        d = docs_or_packed[i] if isinstance(docs_or_packed, list) else docs_or_packed[src[i]:src[i + 1]]
        arr[int(off[i]):int(off[i]) + d.size] = d
    return buf, arr


def test_padded_batch_overlapped(cj, oracle, ctx):
    """A batch already in the device layout, copied in chunks while the scan
    runs: every document's result and verdict as the oracle's, and the same
    as the packed path's."""
    docs = mixed_docs(cj, seed=10)
    sizes = [d.size for d in docs]
    buf, arr = padded_copy(cj, docs, sizes)
    ctx.parse_batch_padded(arr, sizes)
    check_batch(cj, oracle, docs, ctx.batch_results())
    first = ctx.batch_layout()[0].copy()
    ctx.stage_batch_packed(np.concatenate(docs), sizes)
    ctx.run()
    np.testing.assert_array_equal(ctx.batch_layout()[0], first)
    buf.close()


def test_padded_batch_full_size(cj, ctx):
    """Config 4 (4096 documents, 2 GiB, 1 % invalid UTF-8, 1 % bad brackets)
    through the overlapped padded path: identical to the packed graph path."""
    packed, sizes, kinds = synth.batch_input(synth.CONFIG_SEED_BASE + 4, 4096, 2 << 30)
    ctx.stage_batch_packed(packed, sizes)
    ctx.run_graph()
    want, wst, wS, wd, woff = ctx.batch_layout()
    want = want.copy()
    buf, arr = padded_copy(cj, packed, sizes)
    ctx.parse_batch_padded(arr, sizes)
    got, st, S, d, off = ctx.batch_layout()
    np.testing.assert_array_equal(st, wst)
    np.testing.assert_array_equal(S, wS)
    np.testing.assert_array_equal(off, woff)
    np.testing.assert_array_equal(got[:int(off[-1])], want[:int(woff[-1])])
    assert int((st != cj.OK).sum()) == int((kinds > 0).sum())
    buf.close()
