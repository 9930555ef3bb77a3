import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "micromagnetic-gpu-monte-carlo_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def M():
    """The libmmc ctypes binding (builds libmmc.so first if needed)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("mmc_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import mmc_ctypes
    mmc_ctypes.lib()
    return mmc_ctypes


@pytest.fixture(scope="session")
def O():
    """The CPU oracle (test infrastructure)."""
    import oracle_ctypes
    oracle_ctypes.lib()
    return oracle_ctypes
