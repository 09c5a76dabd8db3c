import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long-running (rollouts)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libsph2s.so and the oracle in-tree once per session."""
    from oracle.build import build_oracle
    from sph2s_final_gb300.build import build_library
    build_library()
    build_oracle()
    yield
