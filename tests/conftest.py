import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "multiple-double-arithmetic-matrix-matrix-multiplication_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def pkg(sub=None):
    """Import the library package (its directory name has hyphens)."""
    name = PKG_NAME if sub is None else PKG_NAME + "." + sub
    return importlib.import_module(name)


@pytest.fixture(scope="session")
def inputs():
    return pkg("inputs")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build(ref=False)
    return oracle


GOLDEN = os.path.join(ROOT, "tests", "golden")
