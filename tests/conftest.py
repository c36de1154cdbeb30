import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libsphnj on the device)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """libsphnj.so (host part usable without a GPU) and the oracle."""
    import oracle
    import sphnj_gb300

    sphnj_gb300.build()
    oracle.build()
    yield
