import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libswgb300.so")


@pytest.fixture(scope="session")
def sw():
    import __graft_entry__

    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as o

    o.load()
    return o
