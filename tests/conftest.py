import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")
    config.addinivalue_line("markers", "slow: CPU test that takes more than ~10 s")


@pytest.fixture(scope="session")
def engine():
    """One engine context for the GPU tests (fails loudly without a GPU)."""
    from pbig_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()
