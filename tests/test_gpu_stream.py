"""Streamed one-shot parses (cj_parse_into with pinned input and pinned output
of at least 256 MiB): the input's copy, the scan in waves and the copy of each
wave's positions back to the host overlap.  Bit-exact against the oracle and
against the staged path, for standard JSON and JSON Lines; capacity and
validation errors as the non-streamed path reports them."""
import numpy as np
import pytest

from tests import synth

pytestmark = pytest.mark.gpu

STREAM_MIN = 256 << 20


def pinned_copy(cj, data):
    buf = cj.PinnedBuffer(data.size)
    buf.array[:] = data
    return buf


def parse_streamed(cj, ctx, data, lines=False, cap=None):
    src = pinned_copy(cj, data)
    n = cap if cap is not None else 2 * data.size + 4
    out = cj.PinnedBuffer(4 * n, dtype=np.int32)
    try:
        inf = ctx.parse_into(src.array, out.array, lines=lines)
        return inf, out.array[:2 * inf.n_structural + 4].copy()
    finally:
        src.close()
        out.close()


@pytest.mark.parametrize("extra", [0, 12345, (64 << 20) + 3])
def test_standard(cj, ctx, oracle, extra):
    d = synth.synth_document(0x57AE0 + extra, STREAM_MIN + extra, max_depth=14, huge_string_frac=0.02,
                             huge_string_min=20000, huge_string_max=200000)
    ref = oracle.parse(d)
    assert ref.flags == 0
    inf, out = parse_streamed(cj, ctx, d)
    assert inf.status == 0 and inf.n_structural == ref.n_structural
    np.testing.assert_array_equal(out, ref.reference_layout())


def test_lines(cj, ctx, oracle):
    d, _ = synth.synth_lines(0x57AE1, STREAM_MIN + 4099)
    ref = oracle.parse(d, lines=True)
    assert ref.flags == 0
    inf, out = parse_streamed(cj, ctx, d, lines=True)
    assert inf.n_structural == ref.n_structural
    np.testing.assert_array_equal(out, ref.reference_layout())
    # the same bytes staged and run in one scan
    res = ctx.parse_json_lines([d])
    np.testing.assert_array_equal(res.buffer, out)


def test_backslash_string(cj, ctx, oracle):
    """One string of backslash runs across every wave boundary."""
    d = synth.synth_backslash_string(0x57AE2, STREAM_MIN + 777)
    ref = oracle.parse(d)
    inf, out = parse_streamed(cj, ctx, d)
    assert inf.n_structural == ref.n_structural
    np.testing.assert_array_equal(out, ref.reference_layout())


def test_capacity_and_errors(cj, ctx, oracle):
    d = synth.synth_document(0x57AE3, STREAM_MIN, max_depth=8)
    ref = oracle.parse(d)
    with pytest.raises(cj.CujsonError) as e:
        parse_streamed(cj, ctx, d, cap=ref.n_structural)          # room for the positions only
    assert e.value.status == cj.ERR_CAPACITY
    for kind, status in ((1, cj.ERR_INVALID_UTF8), (4, cj.ERR_INVALID_BRACKETS)):
        bad = d.copy()
        assert synth.synth_corrupt(bad, kind, 11)
        with pytest.raises(cj.CujsonError) as e:
            parse_streamed(cj, ctx, bad)
        assert e.value.status == status
    # the context parses normally afterwards, staged and streamed
    inf, out = parse_streamed(cj, ctx, d)
    np.testing.assert_array_equal(out, ref.reference_layout())
    np.testing.assert_array_equal(ctx.parse_standard_json(d).buffer, out)
