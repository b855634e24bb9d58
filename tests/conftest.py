import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build (if stale) the CUDA library and the CPU oracle before any test."""
    from blochlib_gb300 import build
    build.build_library()
    build.build_examples()
    build.build_oracle()
    yield
