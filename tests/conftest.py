import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "genericschur.jl_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def gs():
    """The CUDA library's Python host package, built in-tree for sm_103a."""
    import build_lib
    build_lib.build()
    import genericschur_gb300
    return genericschur_gb300
