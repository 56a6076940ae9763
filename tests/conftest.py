import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
# a fatal signal in the library's threads prints their native frames (reffine_gb300 crash report)
os.environ.setdefault("RF_CRASH_TRACE", "1")
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    """The backend library is built in-tree (incremental: a no-op when up to date)."""
    from reffine_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def eng():
    from reffine_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()
