import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def iris():
    return importlib.import_module("irisfdtd-academic_gb300")


@pytest.fixture(scope="session")
def oracle():
    import iris_oracle
    iris_oracle.build()
    return iris_oracle


def golden(name):
    return os.path.join(GOLDEN, name)
