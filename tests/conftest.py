import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libtnad.so")
    config.addinivalue_line("markers", "slow: long-running CPU oracle case")


@pytest.fixture(scope="session")
def tn():
    """The package (libtnad host mirror); builds libtnad.so if missing."""
    import __graft_entry__ as ge

    lib = ge.PKG_DIR / "libtnad.so"
    if not lib.exists():
        ge.build()
    return ge.load_package()


@pytest.fixture(scope="session")
def orc():
    from oracle import tnad_oracle

    return tnad_oracle
