import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built libfftdock.so")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_lib():
    """Path of libfftdock.so; builds it in-tree if it is missing."""
    from proddl2_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        from proddl2_gb300 import build
        build.build()
    return _lib.LIB_PATH
