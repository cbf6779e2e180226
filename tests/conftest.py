import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native libraries in-tree if they are missing (the GPU machine
    builds them before the tests; this makes a fresh checkout testable)."""
    from spacelab_gb300 import build
    if not build.LIB.exists() or not build.ORACLE_LIB.exists():
        build.build_all()
    yield
