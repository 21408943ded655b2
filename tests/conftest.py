import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def ib():
    import __graft_entry__ as ge
    return ge.package()


@pytest.fixture(scope="session")
def O():
    from oracle import ib_oracle
    return ib_oracle


@pytest.fixture(scope="session")
def lib(ib):
    import __graft_entry__ as ge
    ge.build()
    return ib.load_library()
