import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; fails loudly otherwise."""
    from simcoflow3d_gb300 import build
    build.build()
    from simcoflow3d_gb300 import projection
    return projection.load_library()
