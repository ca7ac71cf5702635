"""Builds tests/dropin/_build/iter_std and iter_lines: tests/dropin/iter_driver.cpp
compiled against the drop-in iterator header include/cujson/cujson_iter.h."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
BUILD = HERE / "_build"
DRIVER = HERE / "iter_driver.cpp"
HEADERS = [REPO / "include" / "cujson" / "cujson_iter.h", REPO / "include" / "cujson" / "cujson_types.h",
           REPO / "include" / "cujson_gb300.h"]


def build(force: bool = False) -> dict:
    BUILD.mkdir(parents=True, exist_ok=True)
    newest = max(p.stat().st_mtime for p in [DRIVER, *HEADERS])
    out = {}
    for name, lines in (("iter_std", 0), ("iter_lines", 1)):
        exe = BUILD / name
        if force or not exe.exists() or exe.stat().st_mtime < newest:
            cmd = ["g++", "-std=c++17", "-O2", "-Wall", f"-I{REPO / 'include'}",
                   f"-DCJ_ITER_LINES={lines}", str(DRIVER), "-o", str(exe)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"iterator driver build failed:\n{r.stderr}")
        out[name] = exe
    return out


if __name__ == "__main__":
    print(build(force=True))
