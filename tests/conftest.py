import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def built_lib():
    """The GPU library, built if needed; the GPU tests go through it only."""
    from traffic_assignment_gb300 import build as b
    import traffic_assignment_gb300 as tg

    b.build()
    return tg.load_library()


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN
