"""Shared test setup: the `gpu` marker, the package handle and the oracle."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def jx():
    return importlib.import_module("sycl-jaccard_gb300")


@pytest.fixture(scope="session")
def O():
    from oracle import oracle
    return oracle
