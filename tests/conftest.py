import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG = "texture-synthesis_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def ts():
    """The product package, with libtsgpu.so built (fails loudly otherwise)."""
    importlib.import_module(PKG + ".build").build()
    mod = importlib.import_module(PKG)
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def wl():
    return importlib.import_module(PKG + ".workloads")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o

    o.lib()
    return o
