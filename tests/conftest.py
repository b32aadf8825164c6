import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def blob():
    from mima_gb300 import tables
    return tables.ensure_blob()


@pytest.fixture(scope="session")
def orc(blob):
    from oracle import oracle as o
    o.load(blob)
    o.set_table_mode(True)
    return o


@pytest.fixture(scope="session")
def gpu(blob):
    """One GPU handle for the session; fails loudly if the library or GPU is missing."""
    from mima_gb300 import rrtmg
    r = rrtmg.RRTMG(blob)
    yield r
    r.close()


def rel_err(a, b, floor):
    import numpy as np
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))
