import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libchgpu.so")


@pytest.fixture(scope="session")
def oracle_mod():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds libchgpu.so if needed and loads it; GPU tests only."""
    from channel_gb300 import build as b
    from channel_gb300 import lib

    b.build()
    return lib.load_library()


def rel_l2(a, b):
    import numpy as np

    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
