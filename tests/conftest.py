"""Shared test setup: repository root on sys.path, the `gpu` marker, and
session fixtures that build the oracle (the checker) and the CUDA library."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    O.lib()
    return O


@pytest.fixture(scope="session")
def e2d():
    """The CUDA library wrapper; builds the library when it is missing."""
    import euler2d_cudafortran_gb300 as E
    from euler2d_cudafortran_gb300 import build
    if not all(os.path.exists(p) for p in E.LIB_PATHS.values()):
        build.build()
    E.load_library()
    return E
