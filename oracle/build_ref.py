"""Recipe that compiles parts of the reference itself, from its sources where
they lie, into oracle/_ref/ -- TEST INFRASTRUCTURE ONLY.

What it builds (each only when the reference tree is present):

* iter_ref_std, iter_ref_lines -- tests/dropin/iter_driver.cpp compiled with
  g++ against the reference's own query iterators
  (cujson/query/query_iterator_standard_json.cpp and query_iterator.cpp,
  prepended with -include).  The iterators are plain host C++; cudaFreeHost
  is the only CUDA call they make and the driver never reaches it, so they run
  on a machine without a GPU and give the golden query answers under
  tests/golden/.

The reference's parse path is CUDA + Thrust and needs a GPU, and the reference
tree is not available where a GPU is, so its parse outputs are not built here.

usage: python oracle/build_ref.py [reference root]
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
OUT = HERE / "_ref"
DRIVER = REPO / "tests" / "dropin" / "iter_driver.cpp"
DEFAULT_REF = Path(os.environ.get("CUJSON_REFERENCE", "/root/reference"))
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def iter_targets(ref: Path):
    q = ref / "cujson" / "query"
    return {
        "iter_ref_std": (q / "query_iterator_standard_json.cpp", 0),
        "iter_ref_lines": (q / "query_iterator.cpp", 1),
    }


def build(ref: Path = DEFAULT_REF, force: bool = False) -> dict:
    """Build what the reference tree allows; returns {name: path}."""
    if not (ref / "cujson" / "query").is_dir():
        return {}
    OUT.mkdir(parents=True, exist_ok=True)
    built = {}
    for name, (src, lines) in iter_targets(ref).items():
        exe = OUT / name
        newest = max(DRIVER.stat().st_mtime, src.stat().st_mtime)
        if force or not exe.exists() or exe.stat().st_mtime < newest:
            cmd = ["g++", "-std=c++17", "-O1", "-w", f"-I{CUDA_HOME / 'include'}",
                   "-DCJ_ITER_REF=1", f"-DCJ_ITER_LINES={lines}", "-include", "cuda_runtime.h",
                   "-include", str(src),
                   str(DRIVER), "-o", str(exe), f"-L{CUDA_HOME / 'lib64'}", "-lcudart",
                   f"-Wl,-rpath,{CUDA_HOME / 'lib64'}"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference iterator build failed:\n{r.stderr}")
        built[name] = exe
    return built


if __name__ == "__main__":
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF
    for k, v in build(ref, force=True).items():
        print(k, v)
