import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "fluid-simulation_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and libfluidgb.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    orc.load()
    return orc


@pytest.fixture(scope="session")
def fluidlib():
    """libfluidgb.so (built here if missing, so the symbol checks run on CPU too)."""
    from fluidgb import build
    from fluidgb import _abi
    if not os.path.exists(_abi.LIB_PATH):
        build.build()
    return _abi.load_library()
