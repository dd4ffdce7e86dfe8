import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def sv():
    """The package with its library built (GPU tests)."""
    import __graft_entry__ as ge
    ge._build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def ctx(sv):
    c = sv.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def O():
    from oracle import severo_oracle
    return severo_oracle
