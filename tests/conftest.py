import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def golden():
    import numpy
    return dict(numpy.load(os.path.join(ROOT, "tests", "golden", "reference_golden.npz")))
