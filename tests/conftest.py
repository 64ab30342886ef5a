import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

# mount point of the reference sources (read only); tests that need them skip
# where it is absent
REFERENCE = os.environ.get("FVS2D_REFERENCE", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the device path through the C-ABI")


@pytest.fixture(scope="session")
def reference_examples():
    """Directory of the reference's example inputs, when the reference is mounted."""
    d = os.path.join(REFERENCE, "examples")
    if not os.path.isdir(d):
        pytest.skip("reference examples not available on this machine")
    return d
