"""The parse kernels themselves (cujson_gb300/csrc/cj_scan.cu, cj_pair.cu),
compiled for the CPU through the emulation in tests/emu and run the way the
library runs them, against the oracle -- no GPU.  Every buffer the kernels
get ends at a guard page, so an out-of-bounds access stops the test process.

This checks the kernels' own code paths (warp collectives, staging buffers,
prefix composition, the work list, the per-document paths of a batch) before
it runs on a GPU."""
import ctypes

import numpy as np
import pytest

from tests import synth
from tests.emu import build as emu_build


def _load(variant=""):
    L = ctypes.CDLL(str(emu_build.build(variant=variant)))
    L.cje_parse.restype = ctypes.c_int
    L.cje_parse.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int64),
                            ctypes.POINTER(ctypes.c_uint32), ctypes.c_void_p]
    L.cje_parse_batch.restype = ctypes.c_int
    L.cje_parse_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint32),
                                  ctypes.c_void_p, ctypes.c_void_p]
    L.cje_parse_waves.restype = ctypes.c_int
    L.cje_parse_waves.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint32)]
    return L


@pytest.fixture(scope="module")
def emu():
    return _load()


def emu_parse(emu, data, lines=False, chunks=None, region_kib=8, wave_regions=0):
    buf = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8) if isinstance(data, bytes) else data)
    sizes = np.asarray(chunks if chunks is not None else [buf.size], np.uint64)
    cap = buf.size + 1
    pos = np.zeros(cap, np.int32)
    pair = np.zeros(cap, np.int32)
    S = ctypes.c_int64()
    fl = ctypes.c_uint32()
    if wave_regions:
        emu.cje_parse_waves(buf.ctypes.data, sizes.ctypes.data, sizes.size, int(lines), region_kib, wave_regions,
                            pos.ctypes.data, pair.ctypes.data, cap, ctypes.byref(S), ctypes.byref(fl))
    else:
        emu.cje_parse(buf.ctypes.data, sizes.ctypes.data, sizes.size, int(lines), region_kib, pos.ctypes.data,
                      pair.ctypes.data, cap, ctypes.byref(S), ctypes.byref(fl), None)
    return pos[:S.value], pair[:S.value], fl.value


def check(emu, oracle, data, lines=False, chunks=None, region_kib=8, wave_regions=0):
    p, q, fl = emu_parse(emu, data, lines, chunks, region_kib, wave_regions)
    r = oracle.parse(data, lines=lines, chunk_sizes=chunks)
    assert fl & 0x0C == 0, hex(fl)                      # no timeout, no count mismatch
    assert bool(fl & 1) == bool(r.flags & oracle.ERR_UTF8)
    assert bool(fl & 2) == bool(r.flags & oracle.ERR_BRACKETS)
    np.testing.assert_array_equal(p, r.positions)
    if r.flags == 0:
        np.testing.assert_array_equal(q, r.pair_row)


@pytest.mark.parametrize("region_kib", [4, 8, 16])
def test_small_documents(emu, oracle, region_kib):
    for d in (b"[1,2]", b'{"a":"b\\"c,d"}', b'["\\\\",1]', b'["\\\\\\"",1]', b'{"k":[{},[]],"x":{}}',
              b'"[{,:}]"', b"123", b"   ", b"[]", b"{}", b'[[[[{"a":[]}]]]]', b"]]", b"[[[", b"[{]}",
              b"\xc0\x80", b'["\xe2\x82\xac"]'):
        check(emu, oracle, d, region_kib=region_kib)


@pytest.mark.parametrize("n,region_kib", [(1023, 4), (4096, 4), (4097, 8), (8191, 8), (65537, 16),
                                          (300001, 8), (1 << 20, 16)])
def test_generated(emu, oracle, n, region_kib):
    check(emu, oracle, synth.synth_document(n, n, max_depth=12), region_kib=region_kib)


@pytest.mark.parametrize("depth", [1, 300, 5000, 100000])
def test_deep(emu, oracle, depth):
    """Steps of 1024 brackets: every byte a structural."""
    check(emu, oracle, synth.synth_deep(depth))


@pytest.mark.parametrize("seed", range(3))
def test_backslash_runs(emu, oracle, seed):
    check(emu, oracle, synth.synth_backslash_string(seed, 70000 + 4093 * seed), region_kib=[4, 8, 16][seed])


def test_huge_strings(emu, oracle):
    d = synth.synth_document(78, 600000, max_depth=20, huge_string_frac=0.05, huge_string_min=20000,
                             huge_string_max=60000)
    check(emu, oracle, d)


@pytest.mark.parametrize("seed", range(12))
def test_random_bytes(emu, oracle, seed):
    rng = np.random.default_rng(seed)
    alphabet = np.frombuffer(b'[]{}:,"\\ ab\n\xc3\xa9', np.uint8)
    d = alphabet[rng.integers(0, alphabet.size, int(rng.integers(1, 40000)))]
    lines = bool(seed & 1)
    check(emu, oracle, d, lines=lines, region_kib=[4, 8, 16][seed % 3])


@pytest.mark.parametrize("chunks", [1, 3, 7])
def test_json_lines(emu, oracle, cj, chunks):
    d, _ = synth.synth_lines(synth.CONFIG_SEED_BASE + 3, 400000)
    check(emu, oracle, d, lines=True, chunks=cj.plan_lines_count(d, chunks), region_kib=4)


def test_batch(emu, oracle):
    """Independent documents of every size class, valid and invalid, in one
    run: per-document arrays and verdicts."""
    docs = [np.frombuffer(b, np.uint8).copy() for b in (
        b"1", b"[]", b'{"a":"b\\"c,d"}', b"[[[", b"[1,[2]]", b"]]", b"{}", b"[{]}", b"[]",
        b'"\\\\"', b"   ", b'{"k":[{},[]],"x":{}}', b"\xc0\x80", b'["\xed\xa0\x80"]')]
    for k, n in enumerate([1023, 1024, 1025, 4095, 65536, 114689]):
        docs.append(synth.synth_document(700 + k, n, max_depth=10))
    docs.append(synth.synth_deep(20000))
    docs.append(synth.synth_backslash_string(7, 30000))
    sizes = np.array([d.size for d in docs], np.uint64)
    packed = np.concatenate(docs)
    cap = packed.size + len(docs)
    pos = np.zeros(cap, np.int32)
    pair = np.zeros(cap, np.int32)
    S = ctypes.c_int64()
    fl = ctypes.c_uint32()
    dfl = np.zeros(len(docs), np.uint32)
    dS = np.zeros(len(docs), np.int64)
    emu.cje_parse_batch(packed.ctypes.data, sizes.ctypes.data, sizes.size, 8, pos.ctypes.data, pair.ctypes.data,
                        cap, ctypes.byref(S), ctypes.byref(fl), dfl.ctypes.data, dS.ctypes.data)
    assert fl.value & 0x0C == 0
    o = 0
    for i, d in enumerate(docs):
        r = oracle.parse(d)
        assert bool(dfl[i] & 1) == bool(r.flags & oracle.ERR_UTF8), i
        if r.flags == 0:
            assert dfl[i] == 0 and dS[i] == r.n_structural, i
            np.testing.assert_array_equal(pos[o:o + dS[i]], r.positions, err_msg=f"doc {i}")
            np.testing.assert_array_equal(pair[o:o + dS[i]], r.pair_row, err_msg=f"doc {i}")
        elif r.flags & oracle.ERR_BRACKETS:
            assert dfl[i] & 2, i
        o += int(dS[i])


@pytest.mark.parametrize("lines", [False, True])
def test_multi_block_prefix(emu, oracle, cj, lines):
    """1280 regions, 5 prefix blocks: prefix_reduce's block aggregates, and
    each block's run of the aggregates before it."""
    L = emu
    if lines:
        d, _ = synth.synth_lines(synth.CONFIG_SEED_BASE + 3, 5 << 20)
        check(L, oracle, d, lines=True, chunks=cj.plan_lines_count(d, 3), region_kib=4)
    else:
        d = synth.synth_document(0x601D7777, (5 << 20) + 12345, max_depth=12, huge_string_frac=0.02,
                                 huge_string_min=20000, huge_string_max=90000)
        check(L, oracle, d, region_kib=4)


@pytest.mark.parametrize("wave_regions", [1, 3, 256, 300, 600])
@pytest.mark.parametrize("lines", [False, True])
def test_waves(emu, oracle, cj, lines, wave_regions):
    """The scan in waves of regions, each wave starting from the previous
    wave's end value (a streamed parse): the same result as one scan, with wave
    boundaries inside strings, escapes and JSON-Lines records, and waves of
    more than one prefix block."""
    if lines:
        d, _ = synth.synth_lines(synth.CONFIG_SEED_BASE + 13, (2 << 20) + 777)
        check(emu, oracle, d, lines=True, region_kib=4, wave_regions=wave_regions)
        check(emu, oracle, d, lines=True, chunks=cj.plan_lines_count(d, 3), region_kib=4,
              wave_regions=wave_regions)
    else:
        d = synth.synth_document(0x3A7E5, (2 << 20) + 4321, max_depth=12, huge_string_frac=0.05,
                                 huge_string_min=5000, huge_string_max=30000)
        check(emu, oracle, d, region_kib=4, wave_regions=wave_regions)
        b = synth.synth_backslash_string(7, 300000)
        check(emu, oracle, b, region_kib=4, wave_regions=wave_regions)
