import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# the reference checkout (read by fixture generators only; absent on GPU machines)
REFERENCE = os.environ.get("MUON_REFERENCE_DIR", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def lib():
    """The native library, built in-tree if needed (no fallback)."""
    from muon_gb300 import build, native

    build.build()
    return native.load()


def reference_available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "muon"))
