import importlib
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
if str(ROOT / "tests") not in sys.path:
    sys.path.insert(0, str(ROOT / "tests"))

PACKAGE = "iontracks-pulsedproton-python_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def pic():
    """The product package (its directory name is not an identifier)."""
    return importlib.import_module(PACKAGE)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o

    o.build()
    return o
