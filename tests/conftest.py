import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libtlq.so")


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "reference_solutions.npz"))


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libtlq.so; a GPU test without it fails loudly."""
    from tlaloque_gb300 import build as b
    from tlaloque_gb300.tlq import load_library
    b.build()
    return load_library()
