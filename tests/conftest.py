import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    from oracle import build

    build.build_oracle()
    return oracle


def _gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree.  GPU tests fail (not skip) if it cannot load."""
    from mpm_gb300 import build

    build.build()
    from mpm_gb300 import _lib

    return _lib.lib()
