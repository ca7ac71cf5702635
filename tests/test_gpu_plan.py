"""cj_plan_lines_count_device (JSON-Lines chunk plan computed on the device)
against cj_plan_lines_count (the host planner; both are pinned to the
reference's loadJSONLines_chunkCount by tests/test_plan_golden.py), and its
ordering after the stream that fills the buffer."""
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


def test_device_plan_empty(ctx):
    assert ctx.plan_lines_count_device(0, 0, 3) == [0, 0, 0]


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
