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

* refemu_std, refemu_lines -- the reference's parse path itself
  (cujson/utils.cu, cujson/parse_standard_json.cu, cujson/parse_json_lines.cu)
  compiled with g++ for the CPU through the CUDA host emulation in
  oracle/refemu/ (kernels run as fibers, Thrust and the runtime replaced by
  sequential stand-ins), driven by oracle/refemu/driver.cpp.  The only change
  to the reference's text is mechanical and made in a temporary copy: every
  `kernel<<<grid, block>>>(args);` launch becomes a call of the emulator's
  launch function.  Its outputs are the golden parse vectors under
  tests/golden/.

* ref_loader -- the reference's JSON-Lines loaders (cujson/load_file.cu:
  loadJSONLines_chunkCount, _chunkSizeBytes, _chunkSizeMegaBytes) compiled
  unchanged with g++ against the same cuda_runtime.h stand-in, driven by
  oracle/refemu/load_driver.cpp.  Its chunk plans are the golden plans under
  tests/golden/ and the chunk sizes of every JSON-Lines golden case.

usage: python oracle/build_ref.py [reference root]
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
OUT = HERE / "_ref"
DRIVER = REPO / "tests" / "dropin" / "iter_driver.cpp"
# the reference tree: $CUJSON_REFERENCE, else a checkout named "reference"
# beside this repository
DEFAULT_REF = Path(os.environ.get("CUJSON_REFERENCE", str(REPO.parent / "reference")))
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def iter_targets(ref: Path):
    q = ref / "cujson" / "query"
    return {
        "iter_ref_std": (q / "query_iterator_standard_json.cpp", 0),
        "iter_ref_lines": (q / "query_iterator.cpp", 1),
    }


EMU = HERE / "refemu"
LAUNCH = re.compile(r"(\w+)<<<([^<>]+?)>>>\s*\(")


def _in_line_comment(text: str, pos: int) -> bool:
    line_start = text.rfind("\n", 0, pos) + 1
    return "//" in text[line_start:pos]


def _close_paren(text: str, open_pos: int) -> int:
    """Index of the ')' matching text[open_pos] == '(' (comments and strings skipped)."""
    depth, i, n = 0, open_pos, len(text)
    while i < n:
        c = text[i]
        if text.startswith("//", i):
            i = text.find("\n", i)
            if i < 0:
                break
            continue
        if text.startswith("/*", i):
            i = text.find("*/", i) + 2
            continue
        if c in "\"'":
            j = i + 1
            while j < n and text[j] != c:
                j += 2 if text[j] == "\\" else 1
            i = j + 1
            continue
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                return i
        i += 1
    raise ValueError("unbalanced kernel launch")


def rewrite_launches(text: str) -> str:
    """`name<<<g, b>>>(args);` -> `cj_emu::launch(dim3(g), dim3(b), [&] { name(args); });`"""
    out, pos = [], 0
    for m in LAUNCH.finditer(text):
        if m.start() < pos or _in_line_comment(text, m.start()):
            continue
        cfg = [c.strip() for c in m.group(2).split(",")]
        if len(cfg) != 2:
            raise ValueError(f"unexpected launch configuration: {m.group(0)}")
        close = _close_paren(text, m.end() - 1)
        semi = text.index(";", close)
        out.append(text[pos:m.start()])
        out.append(f"cj_emu::launch(dim3({cfg[0]}), dim3({cfg[1]}), [&] {{ {m.group(1)}(")
        out.append(text[m.end():close + 1])
        out.append("; });")
        pos = semi + 1
    out.append(text[pos:])
    return "".join(out)


def build_refemu(ref: Path, force: bool = False) -> dict:
    src_dir = ref / "cujson"
    deps = [EMU / "driver.cpp", EMU / "cj_cuda_emu.h", *sorted((EMU / "shim").rglob("*.h")),
            *sorted((EMU / "shim").rglob("*.cuh")), *sorted(src_dir.glob("*.cu")), *sorted(src_dir.glob("*.h"))]
    newest = max(p.stat().st_mtime for p in deps)
    out = {"refemu_std": OUT / "refemu_std", "refemu_lines": OUT / "refemu_lines"}
    if not force and all(p.exists() and p.stat().st_mtime >= newest for p in out.values()):
        return out
    OUT.mkdir(parents=True, exist_ok=True)
    tmp = Path(tempfile.mkdtemp(prefix="cj_refemu_"))
    try:
        for f in src_dir.glob("*.h"):
            shutil.copy(f, tmp / f.name)
        for f in src_dir.glob("*.cu"):
            (tmp / f.name).write_text(rewrite_launches(f.read_text()))
        for name, lines in (("refemu_std", 0), ("refemu_lines", 1)):
            cmd = ["g++", "-std=c++17", "-O1", "-w", f"-DCJ_REF_LINES={lines}", f"-I{EMU / 'shim'}",
                   f"-I{tmp}", "-x", "c++", str(EMU / "driver.cpp"), "-o", str(out[name])]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference emulation build failed ({name}):\n{r.stderr[-4000:]}")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return out


def build_loader(ref: Path, force: bool = False) -> Path:
    """oracle/_ref/ref_loader: the reference's load_file.cu, as it lies, with
    oracle/refemu/load_driver.cpp."""
    src = ref / "cujson" / "load_file.cu"
    drv = EMU / "load_driver.cpp"
    exe = OUT / "ref_loader"
    newest = max(p.stat().st_mtime for p in (src, drv, EMU / "shim" / "cuda_runtime.h", EMU / "cj_cuda_emu.h"))
    if force or not exe.exists() or exe.stat().st_mtime < newest:
        cmd = ["g++", "-std=c++17", "-O2", "-w", f"-I{EMU / 'shim'}", f"-I{ref / 'cujson'}", str(drv),
               "-o", str(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference loader build failed:\n{r.stderr[-4000:]}")
    return exe


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
    built.update(build_refemu(ref, force))
    built["ref_loader"] = build_loader(ref, force)
    copy_simdjson_sources(ref)
    return built


SIMDJSON_SRC = OUT / "simdjson_src"   # the amalgamation, copied beside the built checkers


def copy_simdjson_sources(ref: Path = DEFAULT_REF) -> bool:
    """Copy the simdjson amalgamation the reference ships
    (paper_reproduced/related_works/simdjson/simdjson.{h,cpp}, Apache-2.0, the
    licence text is in the header) into oracle/_ref/simdjson_src, which is not
    committed but travels with the working tree to machines without the
    reference tree, so that simdjson can be built and timed on their cores.
    False when the reference tree is absent."""
    sj = ref / "paper_reproduced" / "related_works" / "simdjson"
    if not (sj / "simdjson.cpp").is_file():
        return False
    SIMDJSON_SRC.mkdir(parents=True, exist_ok=True)
    for name in ("simdjson.h", "simdjson.cpp"):
        dst = SIMDJSON_SRC / name
        if not dst.exists() or dst.stat().st_mtime < (sj / name).stat().st_mtime:
            shutil.copy2(sj / name, dst)
    return True


def build_simdjson(ref: Path = DEFAULT_REF, force: bool = False):
    """oracle/_ref/simdjson_bench: oracle/simdjson_driver.cpp with the simdjson
    amalgamation the reference ships (paper_reproduced/related_works/simdjson/),
    compiled from the reference tree or, without it, from the copy in
    oracle/_ref/simdjson_src; None when neither exists.  Built on request only
    (timing a related CPU parser, not a checker); the build is for the machine
    it runs on (NEON on Arm, the x86 kernels elsewhere)."""
    sj = ref / "paper_reproduced" / "related_works" / "simdjson"
    if not (sj / "simdjson.cpp").is_file():
        sj = SIMDJSON_SRC
    if not (sj / "simdjson.cpp").is_file():
        return None
    OUT.mkdir(parents=True, exist_ok=True)
    exe = OUT / "simdjson_bench"
    drv = HERE / "simdjson_driver.cpp"
    # an executable copied from another machine is not reused: the stamp names the one it was built on
    stamp = OUT / "simdjson_bench.machine"
    import platform
    here = f"{platform.machine()} {platform.node()}"
    fresh = exe.exists() and stamp.exists() and stamp.read_text() == here and \
        exe.stat().st_mtime >= max(drv.stat().st_mtime, (sj / "simdjson.cpp").stat().st_mtime)
    if force or not fresh:
        cmd = ["g++", "-std=c++17", "-O3", "-DNDEBUG", "-w", f"-I{sj}", str(drv), str(sj / "simdjson.cpp"),
               "-o", str(exe), "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"simdjson build failed:\n{r.stderr[-3000:]}")
        stamp.write_text(here)
    return exe


if __name__ == "__main__":
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF
    for k, v in build(ref, force=True).items():
        print(k, v)
