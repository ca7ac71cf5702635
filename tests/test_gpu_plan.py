"""cj_plan_lines_count_device and cj_plan_lines_bytes_device (JSON-Lines
chunk plans computed on the device) against cj_plan_lines_count and
cj_plan_lines_bytes (the host planners; all are pinned to the reference's
loaders by tests/test_plan_golden.py), and their ordering after the stream
that fills the buffer."""
import numpy as np
import pytest
from tests import synth

pytestmark = pytest.mark.gpu

BLOCK = 65536


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _cases(cj):
    rng = np.random.default_rng(0xC0DE7001)
    lines, _ = synth.synth_lines(synth.CONFIG_SEED_BASE + 3, 8 << 20)
    yield "generated", lines
    yield "open last line", np.concatenate([lines, np.frombuffer(b'{"a":1}', np.uint8)])
    yield "one line, no newline", np.frombuffer(b'{"a":[1,2,3]}', np.uint8)
    yield "only newlines", np.full(200000, ord("\n"), np.uint8)
    yield "empty lines", np.frombuffer(b"\n\n{}\n\n\n[]\n\n", np.uint8)
    for edge in (BLOCK - 2, BLOCK - 1, BLOCK, BLOCK + 1, 3 * BLOCK - 1):
        buf = np.full(4 * BLOCK + 17, ord("x"), np.uint8)
        buf[[edge, edge + 1, 2 * BLOCK, 2 * BLOCK + 5]] = ord("\n")
        yield f"newlines at {edge}", buf
    sparse = np.full(3 << 20, ord("y"), np.uint8)
    sparse[rng.integers(0, sparse.size, 37)] = ord("\n")
    yield "sparse", sparse


def test_device_plan_matches_host_plan(cj, ctx, torch_cuda):
    torch = torch_cuda
    for name, data in _cases(cj):
        d = torch.from_numpy(np.array(data, copy=True)).to("cuda")   # a writable host copy
        for n in (1, 2, 3, 4, 7, 64, 1000):
            want = cj.plan_lines_count(data, n)
            got = ctx.plan_lines_count_device(d.data_ptr(), int(data.size), n)
            assert got == want, (name, n)
            assert sum(got) == data.size, (name, n)


def test_device_bytes_plan_matches_host_plan(cj, ctx, torch_cuda):
    torch = torch_cuda
    for name, data in _cases(cj):
        d = torch.from_numpy(np.array(data, copy=True)).to("cuda")
        for limit in (0, 1, 2, 100, 1023, 1024, 4096, 65536, 1 << 20, data.size - 1, data.size, data.size + 1):
            if limit < 0:
                continue
            want = cj.plan_lines_bytes(data, limit)
            got = ctx.plan_lines_bytes_device(d.data_ptr(), int(data.size), limit)
            assert got == want, (name, limit)
            assert sum(got) == data.size, (name, limit)


def test_device_plan_empty(ctx):
    assert ctx.plan_lines_count_device(0, 0, 3) == [0, 0, 0]
    assert ctx.plan_lines_bytes_device(0, 0, 100) == []


def test_device_plan_waits_for_the_filling_stream(cj, ctx, torch_cuda):
    """The buffer is filled by an asynchronous copy from pinned memory on a
    side stream that is still running when the planner is called with that
    stream: the plan must see the copied bytes, not the zeros before them."""
    torch = torch_cuda
    lines, _ = synth.synth_lines(cj_seed(), 64 << 20)
    want = cj.plan_lines_count(lines, 5)
    host = torch.from_numpy(lines).pin_memory()
    side = torch.cuda.Stream()
    for _ in range(3):
        d = torch.zeros(lines.size, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            torch.cuda._sleep(2_000_000)          # keep the stream busy before the copy
            d.copy_(host, non_blocking=True)
        got = ctx.plan_lines_count_device(d.data_ptr(), int(lines.size), 5, stream=side.cuda_stream)
        assert got == want
        torch.cuda.synchronize()


def cj_seed():
    return synth.CONFIG_SEED_BASE + 3


@pytest.mark.parametrize("mode,n", [("count", 1), ("count", 4), ("count", 37), ("bytes", 1 << 20),
                                    ("bytes", 65536), ("bytes", 10 << 20)])
def test_parse_lines_planned(cj, ctx, oracle, mode, n):
    """One host buffer planned on the device, moved into place and parsed:
    the same result and segment sizes as planning on the host and calling
    cj_parse_lines, and the oracle's."""
    data, _ = synth.synth_lines(synth.CONFIG_SEED_BASE + 23, (96 << 20) + 12345)
    sizes = cj.plan_lines_count(data, n) if mode == "count" else cj.plan_lines_bytes(data, n)
    if mode == "count":
        res = ctx.parse_lines_planned(data, chunk_count=n)
    else:
        res = ctx.parse_lines_planned(data, chunk_bytes=n)
    offs = np.cumsum([0] + sizes[:-1])
    want = ctx.parse_json_lines([data[o:o + s] for o, s in zip(offs, sizes)])
    np.testing.assert_array_equal(res.buffer, want.buffer)
    assert list(res.segment_sizes) == list(want.segment_sizes)
    ref = oracle.parse(data, lines=True, chunk_sizes=sizes)
    np.testing.assert_array_equal(res.buffer, ref.reference_layout())


def test_parse_lines_planned_refuses_empty_chunks(cj, ctx):
    """A first line longer than the byte limit gives an empty first chunk,
    which cj_parse_lines refuses (as parse_json_lines does): so does the
    planned parse; and more chunks than lines."""
    data = np.frombuffer(b"[" + b"1," * 3000 + b"1]\n" + b"{}\n" * 10, np.uint8).copy()
    with pytest.raises(cj.CujsonError) as e:
        ctx.parse_lines_planned(data, chunk_bytes=1000)
    assert e.value.status == cj.ERR_INVALID_ARGUMENT
    with pytest.raises(cj.CujsonError) as e:
        ctx.parse_lines_planned(data, chunk_count=50)
    assert e.value.status == cj.ERR_INVALID_ARGUMENT
    res = ctx.parse_lines_planned(data, chunk_count=3)
    assert res.n_structural > 0
