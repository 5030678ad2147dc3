import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libffs.so")


@pytest.fixture(scope="session")
def pkg():
    return ge.load_package()


@pytest.fixture(scope="session")
def gpu_pkg(pkg):
    """The package with libffs.so built and loaded (GPU tests only)."""
    if not pkg.lib_available():
        ge.build()
    pkg.load()
    return pkg
