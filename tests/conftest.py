import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built_oracle():
    from wumingpic_gb300 import _build
    _build.build_oracle()
    yield


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree; GPU tests fail (not skip) if it cannot be loaded."""
    from wumingpic_gb300 import _build, _lib
    _build.build_library()
    return _lib.lib()
