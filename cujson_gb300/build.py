"""Build recipe for libcujson_gb300.so (in-tree, sm_103a only).

Every translation unit is compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a``) into ``cujson_gb300/_build`` and
linked into one shared library with the C ABI of ``include/cujson_gb300.h``.
A unit is rebuilt only when it, or a header it may include, is newer than its
object file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = BUILD / "libcujson_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _nvcc() -> str:
    return str(_cuda_home() / "bin" / "nvcc")


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.rglob("*.h")))


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or newest_header > t


def _compile(src: Path) -> tuple[Path, str]:
    obj = BUILD / (src.stem + ".o")
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", f"-I{BUILD}", "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd[1:1] = ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the library; returns its path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    # the value decoder's table of powers of five (generated, not committed)
    pow5 = BUILD / "cj_pow5.inc"
    if force or not pow5.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("cj_pow5_table", PKG / "pow5_table.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.write(pow5)
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    srcs = _sources()
    todo = [s for s in srcs if force or _stale(BUILD / (s.stem + ".o"), s, newest_header)]
    if todo:
        with ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
            for obj, log in ex.map(_compile, todo):
                if verbose and log:
                    print(log)
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    if force or todo or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        lib_dir = _cuda_home() / "lib64"
        cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(LIB), *map(str, objs),
               "-Xlinker", f"-rpath,{lib_dir}", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
