import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU case")


@pytest.fixture(scope="session")
def ora():
    from bindings import oracle
    return oracle()


@pytest.fixture(scope="session")
def ref():
    """The reference's own twins; skips where the reference sources are absent."""
    from bindings import reference
    r = reference()
    if r is None:
        pytest.skip("reference twins not built (reference sources absent on this machine)")
    return r


@pytest.fixture(scope="session")
def rv():
    """The product library (host planner works without a GPU)."""
    import revenant_gb300 as rg
    rg.build()
    return rg.lib()


@pytest.fixture(scope="session")
def gpu():
    """A context on the GPU; GPU tests are marked gpu and need a device."""
    import revenant_gb300 as rg
    from revenant_gb300.device import Device
    rg.build()
    return Device()
