import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, required (no skip) for tests marked gpu."""
    from manifoldann_gb300 import _lib

    lib = _lib.load()
    n = _lib.C.c_int32(0)
    _lib.check(lib.mann_device_count(_lib.C.byref(n)))
    assert n.value >= 1, "a gpu test ran without a visible GPU"
    return lib


def load_golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))
