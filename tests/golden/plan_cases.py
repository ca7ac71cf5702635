"""JSON-Lines inputs for the chunk-plan goldens (tests/golden/plan_golden.json):
each case is rebuilt from its name and arguments, deterministically, so only
the plans are stored.  Used by make_plan_golden.py and tests/test_plan_golden.py."""
from __future__ import annotations

import numpy as np

BLOCK = 65536          # the device planner's newline-count block


def _lines_of(lengths, fill=ord("a"), end=b"\n"):
    parts = [bytes([fill]) * max(0, n - len(end)) + end for n in lengths]
    return np.frombuffer(b"".join(parts), np.uint8).copy()


def build(kind: str, args: dict) -> np.ndarray:
    if kind == "generated":
        from tests import synth
        d, _ = synth.synth_lines(args["seed"], args["size"])
        if args.get("open_tail"):
            d = np.concatenate([d, np.frombuffer(b'{"tail":[1,2]}', np.uint8)])
        return d
    if kind == "bytes":
        return np.frombuffer(bytes.fromhex(args["hex"]), np.uint8).copy()
    if kind == "newlines":
        return np.full(args["n"], ord("\n"), np.uint8)
    if kind == "edges":
        buf = np.full(4 * BLOCK + 17, ord("x"), np.uint8)
        e = args["edge"]
        buf[[e, e + 1, 2 * BLOCK, 2 * BLOCK + 5]] = ord("\n")
        return buf
    if kind == "sparse":
        rng = np.random.default_rng(args["seed"])
        buf = np.full(args["size"], ord("y"), np.uint8)
        buf[rng.integers(0, buf.size, args["count"])] = ord("\n")
        return buf
    if kind == "fixed":
        return _lines_of([args["len"]] * args["lines"])
    if kind == "random_lengths":
        rng = np.random.default_rng(args["seed"])
        return _lines_of(rng.integers(1, args["max_len"] + 1, args["lines"]).tolist())
    if kind == "first_long":
        return _lines_of([args["first"]] + [40] * args["lines"])
    if kind == "crlf":
        rng = np.random.default_rng(args["seed"])
        return _lines_of(rng.integers(2, 300, args["lines"]).tolist(), end=b"\r\n")
    raise ValueError(kind)


CASES = [
    ("generated_2m", "generated", dict(seed=0x601D7001, size=2 << 20)),
    ("generated_open_tail", "generated", dict(seed=0x601D7002, size=300000, open_tail=True)),
    ("one_line_no_newline", "bytes", dict(hex=b'{"a":[1,2,3]}'.hex())),
    ("empty_file", "bytes", dict(hex="")),
    ("single_newline", "bytes", dict(hex="0a")),
    ("empty_lines", "bytes", dict(hex=b"\n\n{}\n\n\n[]\n\n".hex())),
    ("only_newlines", "newlines", dict(n=5000)),
    ("first_line_over_limit", "first_long", dict(first=5000, lines=300)),
    ("first_line_over_1m", "first_long", dict(first=(1 << 20) + 7, lines=5000)),
    ("fixed_100", "fixed", dict(len=100, lines=2000)),
    ("random_lengths", "random_lengths", dict(seed=0x601D7003, max_len=3000, lines=1500)),
    ("crlf", "crlf", dict(seed=0x601D7004, lines=3000)),
    ("sparse_3m", "sparse", dict(seed=0x601D7005, size=3 << 20, count=37)),
] + [(f"block_edge_{e}", "edges", dict(edge=e)) for e in (BLOCK - 2, BLOCK - 1, BLOCK, BLOCK + 1, 3 * BLOCK - 1)]

COUNTS = [1, 2, 3, 4, 7, 64, 1000]
BYTE_LIMITS = [0, 1, 64, 100, 199, 200, 201, 4096, 65536, 1 << 20]
MEGABYTES = [1, 2]
