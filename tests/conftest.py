"""Shared fixtures: package modules (the package directory name starts with a
digit, so it is imported through importlib), the oracle (test infrastructure)
and the gpu marker."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

PKG = "2dmaterialsopticalprops_gb300"


def pkg(name: str):
    return importlib.import_module(f"{PKG}.{name}")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def synth():
    return pkg("synth")


@pytest.fixture(scope="session")
def rpa():
    pkg("build").build()
    return pkg("rpa")


@pytest.fixture(scope="session")
def orc():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def npo():
    import np_oracle
    return np_oracle
