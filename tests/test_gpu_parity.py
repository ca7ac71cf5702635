"""GPU parse vs the oracle, through the C ABI (bit-exact; integer outputs)."""
import numpy as np
import pytest
from tests import synth

pytestmark = pytest.mark.gpu


def assert_same(res, ref):
    assert res.n_structural == ref.n_structural
    np.testing.assert_array_equal(res.positions, ref.positions)
    np.testing.assert_array_equal(res.pair_row, ref.pair_row)
    np.testing.assert_array_equal(res.buffer, ref.reference_layout())


@pytest.mark.parametrize("doc", [
    b"[1,2]", b'{"a":"b\\"c,d"}', b'["\\\\",1]', b'["\\\\\\"",1]', b'{"k":[{},[]],"x":{}}',
    b'"[{,:}]"', b"123", b"   ", b'[":" , "{" ]', b"[]", b"{}", b'[[[[{"a":[]}]]]]',
])
def test_small(ctx, oracle, doc):
    st, res = ctx.try_parse(doc)
    assert st == 0
    assert_same(res, oracle.parse(doc))


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 255, 7167, 7168, 7169, 8191, 8192, 8193, 16384, 65537,
                               114687, 114688, 114689, 131071, 131072, 131073, 229377, 300001,
                               344064, 1 << 21])
def test_sizes(cj, ctx, oracle, n):
    d = synth.synth_document(n, n) if n >= 2 else np.frombuffer(b"1", np.uint8)
    st, res = ctx.try_parse(d)
    ref = oracle.parse(d)
    assert st == 0 and ref.flags == 0
    assert_same(res, ref)


@pytest.mark.parametrize("seed", range(8))
def test_documents(cj, ctx, oracle, seed):
    n = [5000, 70000, 1 << 20, 3 << 20, 123457, 9999, 2 << 20, 777777][seed]
    d = synth.synth_document(2000 + seed, n, max_depth=10)
    res = ctx.parse_standard_json(d)
    assert_same(res, oracle.parse(d))


def test_huge_strings(cj, ctx, oracle):
    d = synth.synth_document(78, 4 << 20, max_depth=20, huge_string_frac=0.05,
                          huge_string_min=20000, huge_string_max=90000)
    assert_same(ctx.parse_standard_json(d), oracle.parse(d))


@pytest.mark.parametrize("seed", range(3))
def test_backslash_runs(cj, ctx, oracle, seed):
    d = synth.synth_backslash_string(seed, 200000 + 4093 * seed)
    assert_same(ctx.parse_standard_json(d), oracle.parse(d))


@pytest.mark.parametrize("seed", [0xC0DE5005, 11])
def test_backslash_string_32mib(cj, ctx, oracle, seed):
    """The serving workload's adversarial request: one 32 MiB string of
    backslash runs (even runs, escaped quotes), alone, and as one JSON-Lines
    record between ordinary records, cut into 1 and 3 chunks."""
    d = synth.synth_backslash_string(seed, 32 << 20)
    ref = oracle.parse(d)
    assert ref.flags == 0
    assert_same(ctx.parse_standard_json(d), ref)
    recs, _ = synth.synth_lines(seed, 300000)
    assert recs[-1] == ord("\n")
    lines = np.concatenate([recs, d, np.frombuffer(b"\n", np.uint8), recs])
    for chunks in (1, 3):
        sizes = cj.plan_lines_count(lines, chunks)
        st, res = ctx.try_parse(lines, lines=True, chunk_sizes=sizes)
        ref = oracle.parse(lines, lines=True, chunk_sizes=sizes)
        assert st == 0 and ref.flags == 0
        assert_same(res, ref)


@pytest.mark.parametrize("depth", [1, 256, 257, 10000, 100000])
def test_deep(cj, ctx, oracle, depth):
    d = synth.synth_deep(depth)
    res = ctx.parse_standard_json(d)
    assert_same(res, oracle.parse(d))
    assert res.max_depth == depth


@pytest.mark.parametrize("seed", range(32))
def test_random_bytes(cj, ctx, oracle, seed):
    rng = np.random.default_rng(seed)
    alphabet = np.frombuffer(b'[]{}:,"\\ ab\n', np.uint8)
    n = int(rng.integers(1, 60000)) if seed < 16 else int(rng.integers(100000, 700000))
    d = alphabet[rng.integers(0, alphabet.size, n)]
    lines = bool(seed & 1)
    st, res = ctx.try_parse(d, lines=lines)
    ref = oracle.parse(d, lines=lines)
    if ref.flags:
        assert st in (2, 3)
    else:
        assert st == 0
        assert_same(res, ref)


def test_lines(cj, ctx, oracle):
    d, _ = synth.synth_lines(5, 3 << 20)
    nl = np.flatnonzero(d == 10)
    cuts = [0] + [int(nl[i * len(nl) // 4]) + 1 for i in range(1, 4)] + [d.size]
    sizes = [cuts[i + 1] - cuts[i] for i in range(4)]
    res = ctx.parse_json_lines([d[cuts[i]:cuts[i + 1]] for i in range(4)])
    ref = oracle.parse(d, lines=True, chunk_sizes=sizes)
    assert_same(res, ref)
    assert sum(res.segment_sizes) == res.n_structural and len(res.segment_sizes) == 4


@pytest.mark.parametrize("kind,status", [(1, 2), (2, 2), (3, 2), (4, 3), (5, 3)])
def test_invalid(cj, ctx, oracle, kind, status):
    d = synth.synth_document(500 + kind, 200000)
    assert synth.synth_corrupt(d, kind, 3)
    st, res = ctx.try_parse(d)
    assert st == status and res is None


@pytest.mark.parametrize("doc", [b"[}", b"{]", b"[[]", b"[]]", b"][", b"}{{}", b"[{]}", b"]"])
def test_invalid_brackets(ctx, doc):
    st, _ = ctx.try_parse(doc)
    assert st == 3


def test_utf8_cases(ctx, oracle):
    for body, ok in [("é€😀".encode(), True), (b"\xc0\x80", False), (b"\xe0\x80\x80", False),
                     (b"\xed\xa0\x80", False), (b"\xf5\x80\x80\x80", False), (b"\xe2\x82", False),
                     (b"\x80", False), (b"\xc3\x41", False)]:
        for pad in (0, 1, 2, 29, 30, 31, 7165, 7166, 7167, 8189, 8190, 8191, 114685, 114686, 114687,
                    131069, 131070, 131071):
            doc = b"[" + b" " * pad + b'"' + body + b'"]'
            st, _ = ctx.try_parse(doc)
            assert (st == 0) == ok, (body, pad, st)
            # the same bytes as the very end of the input
            doc = b'[""]' + b" " * pad + body
            st, _ = ctx.try_parse(doc)
            assert (st == 0) == (ok and oracle.utf8_valid(doc)), (body, pad, st)


def test_repeat_deterministic(cj, ctx):
    d = synth.synth_document(99, 2 << 20)
    first = ctx.parse_standard_json(d).buffer
    for _ in range(20):
        assert np.array_equal(ctx.parse_standard_json(d).buffer, first)


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_timed_runs_same_result(cj, ctx, oracle, mode):
    """Runs with events at every kernel boundary (1), at the scan's and the
    run's ends only (2) or at the run's ends only (3) -- the kernels launched
    to overlap in 2 and 3 -- give the oracle's result; the phases add up to
    the span."""
    d = synth.synth_document(321, 24 << 20, max_depth=12)
    ref = oracle.parse(d)
    ctx.stage_standard(d)
    ctx.timing(mode)
    for _ in range(4):
        ctx.run()
    scan, pair, spine, runs = ctx.phase_ms()
    tables, prefix, emit, _ = ctx.scan_phase_ms()
    span = ctx.span_ms()
    ctx.timing(0)
    assert runs == 4 and scan > 0 and span >= scan + pair + spine - 1e-3
    assert pair > 0 if mode != 3 else pair < 0.02
    assert abs(tables + prefix + emit - scan) < 0.01
    if mode >= 2:                           # back-to-back events: next to nothing between them
        assert spine < 0.02 and prefix < 0.02 and emit < 0.02
    assert_same(ctx.staged_result(), ref)


def test_plain_launches_same_result(cj, ctx, oracle):
    """With the dependent launches off (as the server's slots run) the runs
    give the same results."""
    d = synth.synth_document(322, 8 << 20, max_depth=12)
    ref = oracle.parse(d)
    ctx.set_dependent_launch(False)
    try:
        ctx.stage_standard(d)
        ctx.run()
        assert_same(ctx.staged_result(), ref)
        assert_same(ctx.parse_standard_json(d), ref)
    finally:
        ctx.set_dependent_launch(True)


def test_staged_and_into(cj, ctx, oracle):
    d = synth.synth_document(123, 1 << 20)
    ref = oracle.parse(d)
    ctx.stage_standard(d)
    ctx.run()
    assert_same(ctx.staged_result(), ref)
    out = np.zeros(2 * ref.n_structural + 4, np.int32)
    inf = ctx.parse_into(d, out)
    assert inf.n_structural == ref.n_structural
    np.testing.assert_array_equal(out, ref.reference_layout())


def test_empty_input_rejected(ctx):
    st, _ = ctx.try_parse(b"")
    assert st == 1


def _run_doc(pad, runs):
    """A document whose string holds backslash runs of the given lengths, each
    followed by a byte it may escape and separated by in-string text with
    structural bytes; odd runs escape the quote after them."""
    body = b""
    for k, L in enumerate(runs):
        body += b"\\" * L + (b'"x' if L % 2 else b"") + b"t{,}:[" * (k % 3)
    return b"[" + b" " * pad + b'"' + body + b'",{"k":[1,{"v":"\\\""}]}]'


@pytest.mark.parametrize("pad", [0, 1, 30, 31, 32, 511, 1022, 1023, 7167, 114687])
def test_backslash_run_alignments(ctx, oracle, pad):
    """Backslash runs starting and ending on and around 32-byte lane, 1 KiB
    step, 7 KiB region and 112 KiB tile boundaries, even and odd: the steps
    made only of backslashes are skipped by the scan (the escape carry passes
    through), and the ones around them must still resolve every escape."""
    for runs in ([1024], [1023], [1025], [2048], [2047], [3072, 1], [4096, 2, 4095],
                 [7168], [7169], [7167, 1024, 1023], [114688], [114689, 3], [1 << 18, 1 << 18 | 1]):
        doc = _run_doc(pad, runs)
        st, res = ctx.try_parse(doc)
        ref = oracle.parse(doc)
        assert st == 0 and ref.flags == 0, (pad, runs)
        assert_same(res, ref)


def test_input_wait_timeout_reported(cj, ctx, oracle):
    """A bounded wait that runs out: the scan waits for input bytes that a
    counter nobody raises never reports; the kernel gives up after a few polls,
    finishes with its timeout flag, and the context parses normally afterwards."""
    import ctypes
    d = synth.synth_document(4242, 300001)
    ctx.stage_standard(d)
    info = cj.ParseInfo()
    st = cj.lib().cj_run_staged_starved(ctx.handle, 64, ctypes.byref(info))
    assert st == cj.ERR_TIMEOUT and info.error_flags & 0x4
    assert (info.error_flags >> 16) & 0xFF == 6      # the wait for input bytes expired
    st2, res = ctx.try_parse(d)
    assert st2 == cj.OK
    np.testing.assert_array_equal(res.buffer, oracle.parse(d).reference_layout())


def test_result_buffers_kept_and_reused(cj, ctx, oracle):
    """A freed result buffer is kept pinned and handed out again (pinning a
    large buffer costs more than filling it); the results stay exact."""
    d = synth.synth_document(0x9001, 8 << 20)
    ref = oracle.parse(d)
    cj.lib().cj_host_pool_trim()
    for _ in range(3):
        assert_same(ctx.parse_standard_json(d), ref)
    kept = cj.lib().cj_host_pool_trim()
    assert kept >= 4 * (2 * ref.n_structural + 4)
    assert cj.lib().cj_host_pool_trim() == 0
