import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built liblsh.so")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu_lib():
    """Build liblsh.so (sm_103a) and require a CUDA device."""
    from landslidehysea_gb300 import build as B
    from landslidehysea_gb300 import solver
    B.build()
    lib = solver.load()
    if lib.lsh_check_device() != 0:
        pytest.fail("no CUDA device visible to liblsh.so")
    return lib
