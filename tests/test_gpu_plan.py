"""cj_plan_lines_count_device (JSON-Lines chunk plan computed on the device)
against cj_plan_lines_count (the host planner, whose chunk boundaries other
tests pin to the reference's loadJSONLines_chunkCount rule)."""
import numpy as np
import pytest

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
    lines, _ = cj.synth_lines(cj.CONFIG_SEED_BASE + 3, 8 << 20)
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
