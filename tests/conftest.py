import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle.lib()


@pytest.fixture(scope="session")
def engine():
    """Build (if stale) and load the CUDA engine; GPU tests fail loudly without it."""
    import torch
    from impec2d_gb300 import build as B
    B.build()
    import impec2d_gb300 as E
    E.lib()
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return E
