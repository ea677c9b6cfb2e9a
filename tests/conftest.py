import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the package, the repository root (oracle/) and tests/ (shared references
# such as fsai_reference)
for p in (os.path.join(ROOT, "warp-mfem_gb300"), ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built_lib():
    """Builds libmfem_gb300.so if it is missing or stale (nvcc cross-compiles
    without a GPU) and returns the loaded ctypes library."""
    from mfem_gb300 import build, _lib
    try:
        build.build()
    except RuntimeError as e:  # no nvcc on this machine
        pytest.skip(f"cannot build libmfem_gb300: {e}")
    return _lib.load()
