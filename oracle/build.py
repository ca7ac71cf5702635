"""Build recipe for the oracle: oracle/_build/libcj_oracle.so (gcc, plain C).

Test infrastructure only; see oracle/cj_oracle.h.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libcj_oracle.so"
SRC = [HERE / "cj_oracle.c", HERE / "cj_oracle_query.c"]


def build(force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    newest = max(p.stat().st_mtime for p in SRC + [HERE / "cj_oracle.h"])
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-Wall", "-o", str(LIB),
               *map(str, SRC)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
