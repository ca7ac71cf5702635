"""Builds the sequential CPU model of the kernels (tests/model/cj_model.cpp)."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
LIB = HERE / "_build" / "libcj_model.so"


def build() -> Path:
    LIB.parent.mkdir(exist_ok=True)
    srcs = [HERE / "cj_model.cpp", ROOT / "cujson_gb300" / "csrc" / "cj_device.cuh"]
    if not LIB.exists() or LIB.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{ROOT / 'cujson_gb300' / 'csrc'}",
               "-o", str(LIB), str(HERE / "cj_model.cpp")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(r.stdout + r.stderr)
    return LIB
