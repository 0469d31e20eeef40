import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libatmwfs.so")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle64():
    from oracle.oracle import Oracle
    o = Oracle(64)
    o.set_threads(min(8, os.cpu_count() or 1))
    return o


@pytest.fixture(scope="session")
def oracle32():
    from oracle.oracle import Oracle
    o = Oracle(32)
    o.set_threads(min(8, os.cpu_count() or 1))
    return o


@pytest.fixture(scope="session")
def lib():
    from atmosphericturbulencesimul_gb300 import _lib
    from atmosphericturbulencesimul_gb300.build import build
    build()
    return _lib.load()
