"""Shared pytest configuration: the `gpu` marker and build fixtures."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    from mhm_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def ora_hmath():
    from oracle import oracle
    oracle.build()
    return oracle.load("hmath")


@pytest.fixture(scope="session")
def ora_libm():
    from oracle import oracle
    oracle.build()
    return oracle.load("libm")
