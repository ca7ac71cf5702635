"""Builds the seeded input generators (tests/synth/cj_synth.cpp) into
tests/synth/_build/libcj_synth.so with g++.  Test and benchmark data only:
the parser library does not contain or load it."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libcj_synth.so"
SRC = [HERE / "cj_synth.cpp", HERE / "cj_synth.h"]


def build(force: bool = False) -> Path:
    LIB.parent.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < max(s.stat().st_mtime for s in SRC):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-pthread", f"-I{HERE}",
               "-o", str(LIB), str(HERE / "cj_synth.cpp")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"generator build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
