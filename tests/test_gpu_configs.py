"""The benchmark configurations at full size on the GPU, checked against the
oracle bit for bit (structural positions and pair rows), plus properties that
hold at any size: positions strictly increasing, every pair pointing from an
open to a later close of the same kind, JSON-Lines records split at their
newline entries."""
import numpy as np
import pytest
from tests import synth

pytestmark = pytest.mark.gpu


def check_properties(doc: np.ndarray, res, lines: bool):
    pos = res.positions
    pair = res.pair_row
    S = res.n_structural
    assert np.all(np.diff(pos) > 0)
    chars = doc[pos - 1]
    opens = np.flatnonzero((chars == ord("{")) | (chars == ord("[")))
    closes_at = pair[opens] - 1                      # 0-based structural index of each close
    assert np.all(closes_at > opens) and np.all(closes_at < S)
    want = np.where(chars[opens] == ord("{"), ord("}"), ord("]"))
    assert np.array_equal(chars[closes_at], want)
    nonopen = np.ones(S, bool)
    nonopen[opens] = False
    assert not pair[nonopen].any()
    if lines:
        nl = np.flatnonzero(chars == ord("\n"))
        # every record's brackets close before its newline
        rec_of = np.searchsorted(nl, np.arange(S))
        assert np.array_equal(rec_of[opens], rec_of[closes_at])


def test_config1_64mib(cj, oracle, ctx):
    doc, _ = synth.config_input(1)
    res = ctx.parse_standard_json(doc)
    ref = oracle.parse(doc)
    assert ref.valid
    np.testing.assert_array_equal(res.buffer, ref.reference_layout())
    check_properties(doc, res, False)


def test_config2_1gib(cj, oracle, ctx):
    doc, _ = synth.config_input(2)
    res = ctx.parse_standard_json(doc)
    ref = oracle.parse(doc)
    assert ref.valid
    assert res.n_structural == ref.n_structural
    np.testing.assert_array_equal(res.positions, ref.positions)
    np.testing.assert_array_equal(res.pair_row, ref.pair_row)
    check_properties(doc, res, False)


def test_config3_2gb_lines(cj, oracle, ctx):
    doc, info = synth.config_input(3)
    assert doc.size == cj.MAX_INPUT_BYTES
    sizes = cj.plan_lines_count(doc, 4)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    res = ctx.parse_json_lines([doc[offs[i]:offs[i + 1]] for i in range(len(sizes))])
    ref = oracle.parse(doc, lines=True, chunk_sizes=sizes)
    assert ref.valid
    assert res.n_structural == ref.n_structural
    np.testing.assert_array_equal(res.positions, ref.positions)
    np.testing.assert_array_equal(res.pair_row, ref.pair_row)
    assert res.segment_sizes and sum(res.segment_sizes) == res.n_structural
    check_properties(doc, res, True)
    # every newline byte is a record separator (strings hold no raw newlines)
    assert int((doc[res.positions - 1] == ord("\n")).sum()) == int(np.count_nonzero(doc == ord("\n")))
    assert int(np.count_nonzero(doc == ord("\n"))) >= info["records"]


def test_config4_batch_full(cj, oracle, ctx):
    packed, sizes, kinds = synth.batch_input(synth.CONFIG_SEED_BASE + 4, 4096, 2 << 30)
    ctx.stage_batch_packed(packed, sizes)
    ctx.run_graph()
    layout, status, S, depth, off = ctx.batch_layout()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    assert int((status != cj.OK).sum()) == int((kinds > 0).sum())
    for i in range(sizes.size):
        d = packed[offs[i]:offs[i + 1]]
        ref = oracle.parse(d)
        if kinds[i]:
            assert status[i] != cj.OK and not ref.valid
            continue
        assert status[i] == cj.OK and ref.valid, i
        np.testing.assert_array_equal(layout[off[i]:off[i + 1]], ref.reference_layout(), err_msg=f"doc {i}")


def test_overlapped_copy_pinned(cj, oracle, ctx):
    """One-shot parses of pinned inputs of 64 MiB and more copy the input on a
    second stream while the scan runs; results equal the oracle's and the
    staged (copy-then-run) path's."""
    doc = synth.synth_document(0x0E71A9, (80 << 20) + 12345, max_depth=12)
    pin = cj.PinnedBuffer(doc.size)
    pin.array[:] = doc
    ref = oracle.parse(doc)
    res = ctx.parse_standard_json(pin.array)
    np.testing.assert_array_equal(res.buffer, ref.reference_layout())
    out = np.zeros(2 * ref.n_structural + 4, np.int32)
    info = ctx.parse_into(pin.array, out)
    assert info.status == cj.OK
    np.testing.assert_array_equal(out, ref.reference_layout())
    ctx.stage_standard(doc)
    ctx.run()
    np.testing.assert_array_equal(ctx.staged_result().buffer, res.buffer)
    pin.close()
    lines, _ = synth.synth_lines(0x0E71AA, 96 << 20)
    pl = cj.PinnedBuffer(lines.size)
    pl.array[:] = lines
    sizes = cj.plan_lines_count(lines, 3)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    res = ctx.parse_json_lines([pl.array[offs[i]:offs[i + 1]] for i in range(3)])
    ref = oracle.parse(lines, lines=True, chunk_sizes=sizes)
    np.testing.assert_array_equal(res.positions, ref.positions)
    np.testing.assert_array_equal(res.pair_row, ref.pair_row)
    pl.close()
