"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; the CPU suite
(-m "not gpu") covers the oracle, host logic and the C-ABI surface."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def pkg():
    return graft.load_package()


@pytest.fixture(scope="session")
def oracle():
    oc = graft.load_oracle()
    oc.build()
    return oc


@pytest.fixture(scope="session")
def built(pkg):
    pkg.build.build_all()
    return pkg


@pytest.fixture(scope="session")
def engine(built):
    eng = built.Engine(0)
    yield eng
    eng.close()
