import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")
    # the kernel autotuner's cache of this test session: a file of its own
    import tempfile
    os.environ.setdefault("MFEM_GB300_TUNE_CACHE",
                          os.path.join(tempfile.mkdtemp(prefix="mfem_tune_"), "tune.txt"))


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library (compiled in-tree if missing)."""
    from mfem_gb300.build import build
    from mfem_gb300 import _lib
    build()
    return _lib.load()
