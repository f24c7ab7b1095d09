import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load the CUDA library; GPU tests fail loudly if it is absent."""
    from geoflood_gb300 import build

    build.build()
    from geoflood_gb300 import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def ctx(gpu_lib):
    import geoflood_gb300 as gf

    c = gf.Context(0)
    yield c
    c.close()
