import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def native():
    """The engine's C ABI (built in-tree if missing)."""
    from gpumap_gb300 import _native

    if not _native.lib_path().exists():
        import __graft_entry__

        __graft_entry__.build()
    return _native


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import session

    session.load()
    return session
