"""Writes cj_pow5.inc, the 128-bit powers of five that the value decoder's
Eisel-Lemire conversion (cujson_gb300/csrc/cj_values.cu) multiplies by: for
every decimal exponent q in [-342, 308], 5^q normalised to 128 bits (its top
bit set) -- truncated for q >= 0, rounded up for q < 0 -- as two 64-bit words,
high first.  (D. Lemire, "Number Parsing at a Gigabyte per Second",
Software: Practice and Experience 51(8), 2021, section 5.)  Run by build.py;
the output goes to the build folder."""
from __future__ import annotations

from pathlib import Path

Q_MIN, Q_MAX = -342, 308
MASK64 = (1 << 64) - 1


def entry(q: int) -> int:
    if q >= 0:
        v = 5 ** q
        while v < (1 << 127):
            v <<= 1
        while v >= (1 << 128):
            v >>= 1
        return v
    p = 5 ** -q
    z = p.bit_length()
    if q >= -27:
        return (1 << (z + 127)) // p + 1
    c = (1 << (2 * z + 128)) // p + 1
    while c >= (1 << 128):
        c >>= 1
    return c


def write(path: Path) -> Path:
    lines = ["// generated by cujson_gb300/pow5_table.py: 128-bit powers of five, q = -342 .. 308"]
    for q in range(Q_MIN, Q_MAX + 1):
        v = entry(q)
        lines.append(f"0x{(v >> 64) & MASK64:016x}ull, 0x{v & MASK64:016x}ull,")
    path.write_text("\n".join(lines) + "\n")
    return path


if __name__ == "__main__":
    import sys
    print(write(Path(sys.argv[1]) if len(sys.argv) > 1 else Path("cj_pow5.inc")))
