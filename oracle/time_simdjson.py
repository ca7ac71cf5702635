"""Times simdjson (the copy the reference ships under
paper_reproduced/related_works/simdjson/) on the benchmark workloads, on the
cores of the machine this runs on -- MEASUREMENT INFRASTRUCTURE ONLY, a CPU
data point beside the GPU parse.  The reference tree, and so simdjson's
sources, exist only where the reference is mounted; the GPU machine has neither,
so this runs on the development machine and its numbers are labelled with
that machine's CPU.

usage: python oracle/time_simdjson.py [threads ...]   (needs the reference tree)
"""
from __future__ import annotations

import json
import os
import platform
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from oracle import build_ref  # noqa: E402
from tests import synth  # noqa: E402  (seeded inputs)


def cpu_name() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def run(exe, path, mode, threads, reps):
    r = subprocess.run([str(exe), str(path), mode, str(threads), str(reps)], capture_output=True, text=True,
                       timeout=600)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    f = r.stdout.split()
    return float(f[4])


def main():
    exe = build_ref.build_simdjson()
    if exe is None:
        sys.exit("reference tree not found")
    nthreads = [int(a) for a in sys.argv[1:]] or [1, os.cpu_count() or 1]
    out = {"cpu": cpu_name(), "cores": os.cpu_count(), "machine": platform.machine(), "results": []}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        docs = [
            ("standard JSON 64 MiB (config 1 generator)", synth.config_input(1)[0], ["dom", "index"]),
            ("standard JSON 1 GiB (config 2 generator)", synth.config_input(2)[0], ["dom", "index"]),
            ("JSON Lines 256 MiB (config 3 generator)", synth.synth_lines(synth.CONFIG_SEED_BASE + 3, 256 << 20)[0],
             ["lines"]),
        ]
        for name, data, modes in docs:
            path = td / "doc.json"
            data.tofile(path)
            for mode in modes:
                for t in nthreads:
                    reps = 3 if data.size > (512 << 20) else 10
                    gbs = run(exe, path, mode, t, reps)
                    out["results"].append({"workload": name, "mode": mode, "threads": t, "GBps": round(gbs, 3)})
                    print(json.dumps(out["results"][-1]), flush=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
