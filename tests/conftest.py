import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def native_lib():
    """Build (if stale) the native library and the oracle before any test."""
    from plugin_navierstokes_gb300 import build

    import oracle

    build.build()
    oracle.build()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from plugin_navierstokes_gb300 import build

    build.build()
    return torch.device("cuda:0")
