"""Builds the CPU emulation of the parse kernels: cujson_gb300/csrc/cj_scan.cu
and cj_pair.cu compiled with g++ against tests/emu/cj_emu.h, with
tests/emu/cj_emu_driver.cpp, into tests/emu/_build/libcj_emu.so.  Test
infrastructure only."""
from __future__ import annotations

import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
CSRC = ROOT / "cujson_gb300" / "csrc"
BUILD = HERE / "_build"
LIB = BUILD / "libcj_emu.so"
UNITS = [CSRC / "cj_scan.cu", CSRC / "cj_pair.cu", CSRC / "cj_values.cu", HERE / "cj_emu_driver.cpp"]
DEPS = UNITS + [HERE / "cj_emu.h", HERE / "shim" / "cuda_runtime.h", CSRC / "cj_device.cuh",
                CSRC / "cj_kernels.h", ROOT / "include" / "cujson_gb300.h"]
FLAGS = ["-O1", "-g", "-std=c++17", "-fPIC", "-w", "-DCJ_EMU=1", f"-I{HERE / 'shim'}", f"-I{CSRC}", f"-I{BUILD}",
         f"-I{ROOT / 'include'}", "-include", str(HERE / "cj_emu.h")]


# Variants of the emulation: extra defines for the kernels' sources, and the
# library each builds.
VARIANTS = {"": []}


def _lib(variant: str) -> Path:
    return LIB if not variant else BUILD / f"libcj_emu_{variant}.so"


def _compile(src: Path, variant: str) -> Path:
    obj = BUILD / (src.stem + (f"_{variant}" if variant else "") + ".o")
    cmd = ["g++", *FLAGS, *VARIANTS[variant], "-x", "c++", "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"emulation build failed for {src.name}:\n{r.stderr[-4000:]}")
    return obj


def build(force: bool = False, variant: str = "") -> Path:
    BUILD.mkdir(exist_ok=True)
    pow5 = BUILD / "cj_pow5.inc"          # the value decoder's table of powers of five
    if not pow5.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("cj_pow5_table", ROOT / "cujson_gb300" / "pow5_table.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.write(pow5)
    lib = _lib(variant)
    newest = max(p.stat().st_mtime for p in DEPS)
    if not force and lib.exists() and lib.stat().st_mtime >= newest:
        return lib
    with ThreadPoolExecutor(3) as ex:
        objs = list(ex.map(lambda u: _compile(u, variant), UNITS))
    r = subprocess.run(["g++", "-shared", "-o", str(lib), *map(str, objs)], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(r.stderr)
    return lib


if __name__ == "__main__":
    print(build(force=True))
