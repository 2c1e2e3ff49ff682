"""Shared test setup: the gpu marker, the built libraries and the synthetic scenes."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds (incrementally) the CUDA library and the oracle."""
    import __graft_entry__ as g
    g.build()
    return True


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as orc
    orc.library()
    return orc


def scene_path(name: str) -> str:
    return os.path.join(ROOT, "narvalengine_gb300", "scenes", name + ".json")
