import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine's kernels")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Build the engine and the oracle once per session if they are missing."""
    from litert_gb300 import build as eng_build
    from oracle import build as orc_build

    if not os.path.exists(eng_build.LIB):
        eng_build.build()
    if not os.path.exists(orc_build.LIB):
        orc_build.build()
    yield
