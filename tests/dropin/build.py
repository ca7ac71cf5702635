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


def build_example(libdir: Path, force: bool = False) -> Path:
    """tests/dropin/example_parse.cu against include/cujson/ and libcujson_gb300."""
    BUILD.mkdir(parents=True, exist_ok=True)
    exe = BUILD / "example_parse"
    src = HERE / "example_parse.cu"
    deps = [src, *HEADERS, REPO / "include" / "cujson" / "cujson_api.h", REPO / "include" / "cujson" / "cujson.h"]
    if force or not exe.exists() or exe.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        cmd = ["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
               f"-I{REPO / 'include'}", str(src), "-o", str(exe), f"-L{libdir}", "-lcujson_gb300",
               "-Xlinker", f"-rpath,{libdir}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"example build failed:\n{r.stderr}")
    return exe
