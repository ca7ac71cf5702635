"""The C-ABI library loads and exports every entry point include/*.h declares
(no GPU calls), and the synthetic generators are deterministic."""
import ctypes
import re
from pathlib import Path

import numpy as np
from tests import synth

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(cj_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_exports(cj):
    L = cj.lib()
    names = declared_functions()
    assert len(names) > 20
    for n in names:
        assert hasattr(L, n), n
        assert n in cj.exported_names(), n


def test_status_strings(cj):
    assert cj.status_string(0) == "ok"
    assert "UTF-8" in cj.status_string(cj.ERR_INVALID_UTF8)


def test_generator_deterministic(cj, oracle):
    a = synth.synth_document(synth.CONFIG_SEED_BASE + 1, 3 << 20, max_depth=6, threads=1)
    b = synth.synth_document(synth.CONFIG_SEED_BASE + 1, 3 << 20, max_depth=6, threads=8)
    assert np.array_equal(a, b)
    r = oracle.parse(a)
    assert r.flags == 0 and r.max_depth <= 8
    assert 0.02 < r.n_structural / a.size < 0.08


def test_generator_lines(cj, oracle):
    d, n = synth.synth_lines(3, 1 << 20)
    assert d[-1] == 10 and n > 1000
    assert oracle.parse(d, lines=True).flags == 0
    sizes = np.diff(np.flatnonzero(np.concatenate([[10], d])[:-1] == 10))
    assert np.median(sizes) > 100


def test_corrupt_kinds(cj, oracle):
    for kind, bit in [(1, oracle.ERR_UTF8), (2, oracle.ERR_UTF8), (3, oracle.ERR_UTF8),
                      (4, oracle.ERR_BRACKETS), (5, oracle.ERR_BRACKETS)]:
        d = synth.synth_document(kind, 20000)
        assert synth.synth_corrupt(d, kind, 9)
        assert oracle.parse(d).flags & bit


def test_no_device_fails_loudly(cj):
    # without a GPU the product raises instead of falling back to the CPU
    try:
        import torch
        if torch.cuda.is_available():
            return
    except Exception:
        pass
    h = ctypes.c_void_p()
    assert cj.lib().cj_context_create(-1, ctypes.byref(h)) == cj.ERR_NO_DEVICE
