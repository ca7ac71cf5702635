import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def cj():
    from cujson_gb300 import build as b
    b.build()
    import cujson_gb300
    cujson_gb300.lib()
    return cujson_gb300


@pytest.fixture(scope="session")
def oracle():
    from oracle import cj_oracle
    cj_oracle.lib()
    return cj_oracle


@pytest.fixture(scope="session")
def ctx(cj):
    c = cj.Context()
    yield c
    c.close()
