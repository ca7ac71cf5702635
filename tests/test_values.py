"""Value decoding (cj_decode_values, cujson_gb300/csrc/cj_values.cu) against
Python's json module, slot by slot: strings unescaped to UTF-8, integers that
fit int64 exact, every other number the correctly rounded double (bit for
bit), literals, and invalid tokens marked invalid.  The reference has no
value decoder (its iterator returns raw bytes), so Python's json.loads is the
check.  The kernels run through the CPU emulation here (tests/emu) and on the
GPU in the tests marked gpu."""
import ctypes
import json
import math
import random
import struct

import numpy as np
import pytest

from tests import synth
from tests.emu import build as emu_build

NONE, STRING, INT, DOUBLE, TRUE, FALSE, NULL, INVALID = range(8)


def slot_texts(data: bytes, positions):
    """Slot 0: before the first structural; slot i: after structural i."""
    n = len(data)
    pos = [int(p) for p in positions]
    out = []
    for i in range(len(pos) + 1):
        a = 0 if i == 0 else pos[i - 1]
        b = n if i == len(pos) else pos[i] - 1
        out.append((a, data[a:max(a, b)]))
    return out


def expected(text: bytes):
    t = text.strip(b" \t\n\r")
    if not t:
        return NONE, None
    if t in (b"NaN", b"Infinity", b"-Infinity"):
        return INVALID, None                       # Python extensions, not JSON
    try:
        v = json.loads(t)
    except (ValueError, UnicodeDecodeError):
        return INVALID, None
    if isinstance(v, str):
        try:
            return STRING, v.encode("utf-8")
        except UnicodeEncodeError:                 # a lone surrogate
            return INVALID, None
    if v is True:
        return TRUE, None
    if v is False:
        return FALSE, None
    if v is None:
        return NULL, None
    if isinstance(v, int):
        if -(1 << 63) <= v < (1 << 63):
            return INT, v
        try:
            return DOUBLE, float(v)
        except OverflowError:                      # past the largest double: infinity
            return DOUBLE, math.inf if v > 0 else -math.inf
    if isinstance(v, float):
        return DOUBLE, v
    return INVALID, None


def check_values(data: bytes, positions, types, nums, lens, strings):
    """Every slot as Python's json reads it; returns the number of slots."""
    texts = slot_texts(data, positions)
    assert len(texts) == len(types)
    for i, (a, text) in enumerate(texts):
        et, ev = expected(text)
        t = int(types[i])
        assert t == et, (i, text, t, et)
        if et == STRING:
            off, ln = int(nums[i]), int(lens[i])
            assert bytes(strings[off:off + ln]) == ev, (i, text)
        elif et == INT:
            assert int(np.int64(nums[i])) == ev, (i, text)
        elif et == DOUBLE:
            want = struct.unpack("<Q", struct.pack("<d", ev))[0]
            assert int(nums[i]) == want, (i, text, struct.unpack("<d", struct.pack("<Q", int(nums[i])))[0], ev)
    return len(texts)


def number_doc(seed: int, n: int) -> bytes:
    """A JSON array of numbers: edge cases, then random doubles (shortest
    round-trip text, and longer digit strings), integers and exponents."""
    rng = random.Random(seed)
    edge = ["0", "-0", "1", "-1", "9223372036854775807", "-9223372036854775808", "9223372036854775808",
            "-9223372036854775809", "123456789012345678901234567890", "1.5", "-2.25e-3", "1e308",
            "1.7976931348623157e308", "1e309", "-1e400", "1e-400", "2.2250738585072014e-308", "0.1", "0.3",
            "3.14159265358979323846264338327950288", "1e23", "8.98846567431158e307", "5e-1", "1E+2", "1e-7",
            "123.456e-10", "0.000000000000000000000000000000000001", "100000000000000000000000",
            "9007199254740993", "9007199254740992.0", "4.35", "0e10", "-0.0", "1.0000000000000002",
            "7.2057594037927933e16", "2.5e-5", "1234567890123456789", "12345678901234567890",
            "0.30000000000000004", "17976931348623157e292", "1e22", "1e-22", "123e-400",
            # subnormals, the least one, and the halfway points around them
            "5e-324", "4.9406564584124654e-324", "2.4703282292062327e-324", "2.4703282292062328e-324",
            "2.2250738585072011e-308", "2.225073858507201136057409796709131975934819546351645648e-308",
            "1e-310", "-3.5e-320", "1.7976931348623158e308", "1.7976931348623159e308",
            # a halfway point written out in full, and a hair to either side
            "9007199254740993", "9007199254740993.0000000000000000000001", "9007199254740992.9999999999999999999",
            "2." + "0" * 800 + "1", "0." + "0" * 400 + "1", "1" + "0" * 400 + "e-400", "1e99999999"]
    vals = list(edge)
    for _ in range(n):
        k = rng.random()
        if k < 0.4:
            vals.append(repr(rng.uniform(-1e6, 1e6) * 10 ** rng.randint(-300, 300)))
        elif k < 0.6:
            digits = "".join(rng.choice("0123456789") for _ in range(rng.randint(1, 40))).lstrip("0") or "0"
            e = rng.randint(-330, 310)
            vals.append(f"{digits[0]}.{digits[1:] or '0'}e{e}")
        elif k < 0.7:
            vals.append(str(rng.randint(-(1 << 63), (1 << 63) - 1)))
        elif k < 0.8:
            vals.append(str(rng.randint(-(1 << 70), 1 << 70)))
        else:
            vals.append(f"{rng.randint(0, 10 ** 9)}.{rng.randint(0, 10 ** 9):09d}")
    return ("[" + ", ".join(vals) + "]").encode()


STRING_DOC = (b'["", "plain", "esc \\" \\\\ \\/ \\b \\f \\n \\r \\t", "\\u00e9\\u20ac\\ud83d\\ude00", '
              b'"\\u0041\\u00", "\\ud800", "\\udc00x", "\\ud800\\u0041", "\\x", "caf\xc3\xa9", '
              b'"tab\there", "\\uD83D\\uDE00 upper", true, false, null, tru, nul, 01, 1., .5, +1, 1e, --1, abc, '
              b'{"k": "v", "n": [1, -2.5e3, {"x": "\\"q\\""}]}, "' + b"\\\\" * 300 + b'x"]')


@pytest.fixture(scope="module")
def emu():
    L = ctypes.CDLL(str(emu_build.build()))
    L.cje_parse_values.restype = ctypes.c_int
    L.cje_parse_values.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint32),
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    return L


def emu_values(emu, data: bytes, lines=False, chunks=None):
    buf = np.frombuffer(data, np.uint8).copy()
    sizes = np.asarray(chunks if chunks is not None else [buf.size], np.uint64)
    cap = buf.size + 2
    types = np.zeros(cap, np.uint8)
    nums = np.zeros(cap, np.uint64)
    lens = np.zeros(cap, np.uint32)
    strings = np.zeros(buf.size + 1, np.uint8)
    counts = np.zeros(8, np.int64)
    pos = np.zeros(cap, np.int32)
    pair = np.zeros(cap, np.int32)
    S = ctypes.c_int64()
    fl = ctypes.c_uint32()
    emu.cje_parse_values(buf.ctypes.data, sizes.ctypes.data, sizes.size, int(lines), ctypes.byref(S),
                         ctypes.byref(fl), types.ctypes.data, nums.ctypes.data, lens.ctypes.data,
                         strings.ctypes.data, counts.ctypes.data, pos.ctypes.data, pair.ctypes.data, cap)
    assert fl.value == 0
    n = S.value + 1
    return pos[:S.value], types[:n], nums[:n], lens[:n], strings, counts


def test_strings_literals_invalid(emu):
    pos, t, nums, lens, strs, counts = emu_values(emu, STRING_DOC)
    check_values(STRING_DOC, pos, t, nums, lens, strs)
    assert counts.sum() == len(t) and counts[STRING] >= 8 and counts[INVALID] >= 10


def test_numbers(emu):
    d = number_doc(7, 4000)
    pos, t, nums, lens, strs, counts = emu_values(emu, d)
    check_values(d, pos, t, nums, lens, strs)
    assert counts[DOUBLE] > 2000 and counts[INT] > 300


def long_strings_doc(seed: int, n: int) -> bytes:
    """Strings of 300-3000 bytes built from every kind of piece (plain text,
    multi-byte UTF-8, each escape, \\u escapes of 1-3 UTF-8 bytes, surrogate
    pairs, backslash runs), so escapes straddle every lane and step boundary;
    a fifth carry one fault (a lone or reversed surrogate, a bad escape or
    hex digit, a raw control character)."""
    rng = random.Random(seed)
    pieces = ["a", "xyz", "caf\u00e9", "\\\"", "\\\\", "\\/", "\\b", "\\f", "\\n", "\\r", "\\t",
              "\\u0041", "\\u00e9", "\\u20AC", "\\uffff", "\\ud83d\\ude00", "\\uD800\\uDFFF",
              "\u00e9", "\u20ac", "\U0001f600", "\\\\\\\\", "\\\\u0041", " "]
    faults = ["\\ud800", "\\udc00", "\\ude00\\ud83d", "\\x", "\\u12G4", "\\u12", "\x01",
              "\\ud83d\\u0041", "\\ud83dx", "\\\x01", "\\\x1f", "\\ "]
    out = []
    for k in range(n):
        parts, size = [], rng.randint(300, 3000)
        while sum(map(len, parts)) < size:
            p = rng.choice(pieces)
            parts.append(p * rng.randint(1, 40) if p in ("a", "\\\\") else p)
        if k % 5 == 4:
            parts.insert(rng.randrange(len(parts) + 1), rng.choice(faults))
        out.append('"' + "".join(parts) + '"')
    return ("[" + ", ".join(out) + "]").encode("utf-8")


LONG_SLOTS_DOC = (b"[" + b" " * 5000 + b"1, \"a\"" + b"\n" * 700 + b", " + b"1" * 400 + b", tru" + b" " * 3000
                  + b"e, 0." + b"0" * 500 + b"1,\t" + b" \r\n" * 300 + b"\"" + b"x" * 900 + b"\"" + b" " * 999
                  + b", -" + b"9" * 330 + b"e-700, 1e" + b"0" * 300 + b"1]" + b" " * 70000)


def test_long_slots(emu):
    """Slots longer than a thread takes: long whitespace runs (the slot after
    the last structural among them), long numbers, a literal split by
    spaces."""
    pos, t, nums, lens, strs, counts = emu_values(emu, LONG_SLOTS_DOC)
    check_values(LONG_SLOTS_DOC, pos, t, nums, lens, strs)
    assert counts[INVALID] == 1 and counts[STRING] == 2 and counts[DOUBLE] == 4


def test_long_strings(emu):
    d = long_strings_doc(3, 120)
    pos, t, nums, lens, strs, counts = emu_values(emu, d)
    check_values(d, pos, t, nums, lens, strs)
    assert counts[STRING] >= 80 and counts[INVALID] >= 20


def halfway_doc(seed: int, n: int) -> bytes:
    """Exact halfway points between neighbouring doubles (normal and
    subnormal), each also nudged by one unit in its last written digit:
    the inputs the exact conversion decides."""
    import decimal
    decimal.getcontext().prec = 1200
    rng = random.Random(seed)
    vals = []
    for _ in range(n):
        bits = rng.randrange(1, 0x7FEFFFFFFFFFFFFF) if rng.random() < 0.8 else rng.randrange(1, 1 << 52)
        x = struct.unpack("<d", struct.pack("<Q", bits))[0]
        y = struct.unpack("<d", struct.pack("<Q", bits + 1))[0]
        mid = (decimal.Decimal(x) + decimal.Decimal(y)) / 2
        t = format(mid, "e")
        vals.append(t)
        mant, exp = t.split("e")
        ulp = decimal.Decimal(1).scaleb(int(exp) - (len(mant) - 2))
        vals.append(format(mid + ulp, "e"))
        vals.append(format(mid - ulp, "e"))
    return ("[" + ", ".join(vals) + "]").encode()


def test_halfway_points(emu):
    d = halfway_doc(5, 300)
    pos, t, nums, lens, strs, counts = emu_values(emu, d)
    check_values(d, pos, t, nums, lens, strs)
    assert counts[DOUBLE] == 900


def test_deferred_list_overflow(emu):
    """More deferred numbers (subnormals) than the list holds: the rest
    are found by the sweep."""
    d = ("[" + ",".join(f"{k % 97 + 1}e-{310 + k % 13}" for k in range(6000)) + "]").encode()
    pos, t, nums, lens, strs, counts = emu_values(emu, d)
    assert 6000 > len(d) // 64 + 1                 # the short list's capacity
    check_values(d, pos, t, nums, lens, strs)
    assert counts[DOUBLE] == 6000


def test_escaped_strings_past_the_list(emu):
    """More escaped strings than the deferred list holds: the rest are
    decoded where they are."""
    d = ("[" + ",".join(f'"a\\n{k}\\u00e9"' for k in range(20000)) + "]").encode()
    pos, t, nums, lens, strs, counts = emu_values(emu, d)
    assert counts[STRING] > len(d) // 64 + 1       # the short list's capacity
    check_values(d, pos, t, nums, lens, strs)


def test_generated_documents(emu):
    d = synth.synth_document(synth.CONFIG_SEED_BASE + 1, 400000, max_depth=6).tobytes()
    pos, t, nums, lens, strs, counts = emu_values(emu, d)
    check_values(d, pos, t, nums, lens, strs)
    assert counts[INVALID] == 0


def test_json_lines_chunks(emu, cj):
    d, _ = synth.synth_lines(synth.CONFIG_SEED_BASE + 3, 300000)
    sizes = cj.plan_lines_count(d, 3)
    data = d.tobytes()
    pos, t, nums, lens, strs, counts = emu_values(emu, data, lines=True, chunks=sizes)
    check_values(data, pos, t, nums, lens, strs)


def _gpu_values(cj, ctx, data: bytes, lines=False):
    buf = np.frombuffer(data, np.uint8)
    if lines:
        ctx.stage_lines(buf, cj.plan_lines_count(buf, 3))
    else:
        ctx.stage_standard(buf)
    ctx.run()
    res = ctx.staged_result()
    types, nums, lens, strs, counts = ctx.decode_values()
    n = check_values(data, res.positions, types, nums, lens, strs)
    assert sum(counts) == n
    for k in range(8):
        assert counts[k] == int((types == k).sum())
    return types, lens


def _random_string(rng) -> str:
    n = rng.choice([0, 1, 3, 10, 40, 200, 300, 700, 2000])
    plain = [c for c in map(chr, range(0x20, 0x7F)) if c not in '"\\']
    out = []
    while len(out) < n:
        k = rng.random()
        if k < 0.5:
            out.append(rng.choice(plain))
        elif k < 0.6:
            out.append(chr(rng.randint(0xA0, 0xD7FF)))
        elif k < 0.65:
            out.append(chr(rng.randint(0x10000, 0x10FFFF)))
        elif k < 0.8:
            out.append(rng.choice(['\\"', "\\\\", "\\/", "\\b", "\\f", "\\n", "\\r", "\\t"]))
        elif k < 0.9:
            out.append("\\u%04x" % rng.choice([rng.randint(0, 0xD7FF), rng.randint(0xE000, 0xFFFF)]))
        elif k < 0.95:
            cp = rng.randint(0x10000, 0x10FFFF) - 0x10000
            out.append("\\u%04X\\u%04x" % (0xD800 + (cp >> 10), 0xDC00 + (cp & 0x3FF)))
        else:
            out.append("\\\\" * rng.randint(1, 50))
    return '"' + "".join(out) + '"'


def _random_number(rng) -> str:
    k = rng.random()
    if k < 0.3:
        return str(rng.randint(-10 ** rng.randint(1, 25), 10 ** rng.randint(1, 25)))
    if k < 0.6:
        return repr(rng.uniform(-1, 1) * 10 ** rng.randint(-320, 308))
    if k < 0.8:
        d = "".join(rng.choice("0123456789") for _ in range(rng.randint(1, 60))).lstrip("0") or "0"
        return (rng.choice(["", "-"]) + d[0] + ("." + d[1:] if len(d) > 1 else "") + "e"
                + str(rng.randint(-400, 400)))
    return rng.choice(["0", "-0", "0.0", "1e-324", "2.4703282292062328e-324", "1.7976931348623157e308", "1e309"])


def _random_value(rng, depth: int) -> str:
    k = rng.random()
    if depth < 4 and k < 0.15:
        return "[" + ", ".join(_random_value(rng, depth + 1) for _ in range(rng.randint(0, 6))) + "]"
    if depth < 4 and k < 0.3:
        return "{" + ", ".join(_random_string(rng) + ": " + _random_value(rng, depth + 1)
                               for _ in range(rng.randint(0, 6))) + "}"
    if k < 0.6:
        return _random_string(rng)
    if k < 0.9:
        return _random_number(rng)
    return rng.choice(["true", "false", "null"])


@pytest.mark.parametrize("seed", range(12))
def test_random_documents(emu, seed):
    """Random documents: strings of every escape and of 0-2000 bytes,
    numbers of up to 60 digits and any exponent, nesting, and sometimes a
    long whitespace tail; standard JSON, then the same values as JSON Lines
    in chunks cut at line ends."""
    rng = random.Random(seed)
    doc = ("[" + ", ".join(_random_value(rng, 0) for _ in range(rng.randint(1, 150))) + "]"
           + " " * rng.choice([0, 1, 5000])).encode()
    pos, t, nums, lens, strs, counts = emu_values(emu, doc)
    check_values(doc, pos, t, nums, lens, strs)
    lines = [("{" + ", ".join(_random_string(rng) + ": " + _random_value(rng, 1)
                              for _ in range(rng.randint(1, 8))) + "}").encode() for _ in range(rng.randint(2, 40))]
    data = b"\n".join(lines) + b"\n"
    ends = np.cumsum([len(x) + 1 for x in lines])
    cuts = sorted(rng.sample(range(1, len(lines)), min(3, len(lines) - 1)))
    sizes = np.diff(np.concatenate([[0], ends[np.array(cuts) - 1], [len(data)]])).tolist()
    pos, t, nums, lens, strs, counts = emu_values(emu, data, lines=True, chunks=sizes)
    check_values(data, pos, t, nums, lens, strs)


@pytest.mark.gpu
def test_gpu_values(cj, ctx):
    _gpu_values(cj, ctx, STRING_DOC)
    _gpu_values(cj, ctx, LONG_SLOTS_DOC)
    _gpu_values(cj, ctx, long_strings_doc(17, 3000))
    _gpu_values(cj, ctx, number_doc(11, 20000))
    _gpu_values(cj, ctx, halfway_doc(13, 2000))
    _gpu_values(cj, ctx, ("[" + ",".join(f"{k % 97 + 1}e-{310 + k % 13}" for k in range(60000)) + "]").encode())
    _gpu_values(cj, ctx, synth.synth_document(synth.CONFIG_SEED_BASE + 1, 8 << 20, max_depth=6).tobytes())
    _gpu_values(cj, ctx, synth.synth_events(synth.CONFIG_SEED_BASE + 5, 4 << 20)[0].tobytes(), lines=True)
    _gpu_values(cj, ctx, synth.synth_lines(synth.CONFIG_SEED_BASE + 3, 4 << 20)[0].tobytes(), lines=True)


@pytest.mark.gpu
def test_gpu_values_long_strings(cj, ctx):
    """Strings of 64-128 KiB (the deferred list), decoded whole."""
    d = synth.synth_document(0xC0DE0002, 3 << 20, max_depth=20, huge_string_frac=0.05,
                             huge_string_min=64 << 10, huge_string_max=128 << 10).tobytes()
    types, lens = _gpu_values(cj, ctx, d)
    assert int(lens.max()) > 32 << 10


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(4))
def test_gpu_random_documents(cj, ctx, seed):
    rng = random.Random(100 + seed)
    doc = ("[" + ", ".join(_random_value(rng, 0) for _ in range(rng.randint(100, 400))) + "]"
           + " " * rng.choice([0, 5000])).encode()
    _gpu_values(cj, ctx, doc)
    lines = b"\n".join(("{" + ", ".join(_random_string(rng) + ": " + _random_value(rng, 1)
                                         for _ in range(rng.randint(1, 8))) + "}").encode()
                        for _ in range(rng.randint(50, 200))) + b"\n"
    _gpu_values(cj, ctx, lines, lines=True)
