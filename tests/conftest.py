import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def built():
    """Builds libgpview.so and the oracle if their sources are newer (no GPU needed)."""
    import __graft_entry__

    __graft_entry__.build()
    import gpview_gb300

    return gpview_gb300


@pytest.fixture(scope="session")
def ctx(built):
    c = built.Context(0)
    yield c
    c.close()
