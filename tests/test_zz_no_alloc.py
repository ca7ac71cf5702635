"""cj_parse_standard_noalloc (scratch in a fixed __device__ array) against the
arena entry point cj_parse_standard, over calls in a row.

Kept in a file that is collected last so that it runs both after every other
test in one process and, alone, in a fresh one.
"""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest
from tests import synth

REPO = Path(__file__).resolve().parent.parent
MAX = 1048576   # CJ_NOALLOC_MAX_BYTES


def test_declared_limit_matches():
    text = (REPO / "include" / "cujson_gb300.h").read_text()
    m = re.search(r"#define CJ_NOALLOC_MAX_BYTES (\d+)ull", text)
    assert m and int(m.group(1)) == MAX


def test_source_allocates_nothing():
    src = (REPO / "cujson_gb300" / "csrc" / "cj_noalloc.cu").read_text()
    code = re.sub(r"//[^\n]*", "", src)
    for call in ("cudaMalloc", "cudaFree", "cudaHostAlloc", "malloc(", "new ", "std::vector"):
        assert call not in code, call


def _noalloc(cj, torch, doc: np.ndarray, out_cap: int):
    d_in = torch.from_numpy(np.ascontiguousarray(doc)).to("cuda")
    d_out = torch.full((out_cap,), -7, dtype=torch.int32, device="cuda")
    info = cj.ParseInfo()
    stream = torch.cuda.current_stream().cuda_stream
    st = cj.lib().cj_parse_standard_noalloc(ctypes.c_void_p(d_in.data_ptr()), doc.size,
                                            ctypes.c_void_p(d_out.data_ptr()), out_cap,
                                            ctypes.byref(info), ctypes.c_void_p(stream))
    return st, info, d_out.cpu().numpy()


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.gpu
def test_noalloc_matches_arena_path_calls_in_a_row(cj, torch_cuda):
    torch = torch_cuda
    ctx = cj.Context()
    try:
        docs = [synth.synth_document(0xA110C001, 300001, max_depth=12),
                synth.synth_document(0xA110C002, MAX, max_depth=20),
                np.frombuffer(b'{"k":[{},[]],"x":{}}', np.uint8).copy(),
                synth.synth_document(0xA110C001, 300001, max_depth=12)]
        for doc in docs:
            want = ctx.parse_standard_json(doc)
            S = want.n_structural
            st, info, out = _noalloc(cj, torch, doc, 2 * doc.size + 4)
            assert st == cj.OK, cj.status_string(st)
            assert info.n_structural == S and info.max_depth == want.max_depth
            np.testing.assert_array_equal(out[:2 * S + 4], want.buffer)
            assert (out[2 * S + 4:] == -7).all()
    finally:
        ctx.close()


@pytest.mark.gpu
def test_noalloc_verdicts_and_limits(cj, torch_cuda):
    torch = torch_cuda
    ctx = cj.Context()
    try:
        bad = synth.synth_document(0xA110C003, 50000)
        assert synth.synth_corrupt(bad, 1, 5)
        st_arena, _ = ctx.try_parse(bad)
        st, info, out = _noalloc(cj, torch, bad, 2 * bad.size + 4)
        assert st == st_arena != cj.OK
        assert info.status == st
        assert (out == -7).all()          # an invalid document writes nothing
        unbalanced = synth.synth_document(0xA110C005, 50000)
        assert synth.synth_corrupt(unbalanced, synth.CORRUPT_UNBALANCED, 6)
        st, info, out = _noalloc(cj, torch, unbalanced, 2 * unbalanced.size + 4)
        assert st == cj.ERR_INVALID_BRACKETS and (out == -7).all()

        # output too small: refused, nothing written
        doc = synth.synth_document(0xA110C004, 20000)
        st, info, out = _noalloc(cj, torch, doc, 8)
        assert st == cj.ERR_CAPACITY
        assert (out == -7).all()

        # over the scratch limit: refused before any work
        big = np.full(MAX + 1, ord(" "), np.uint8)
        st, _, out = _noalloc(cj, torch, big, 16)
        assert st == cj.ERR_TOO_LARGE
        assert (out == -7).all()

        # a valid call right after the refusals
        want = ctx.parse_standard_json(doc)
        st, _, out = _noalloc(cj, torch, doc, 2 * doc.size + 4)
        assert st == cj.OK
        np.testing.assert_array_equal(out[:2 * want.n_structural + 4], want.buffer)
    finally:
        ctx.close()
