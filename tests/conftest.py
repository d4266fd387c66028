"""Shared test configuration: the `gpu` marker, library builds and the oracle."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU case")


def _ensure_built():
    sys.path.insert(0, ROOT)
    import __graft_entry__
    _build = __graft_entry__._build_module()
    if not os.path.exists(_build.LIB):
        _build.build()
    if not os.path.exists(_build.HOSTCHECK):
        _build.build_hostcheck()
    import oracle
    oracle.build()


_ensure_built()


@pytest.fixture(scope="session")
def gl():
    import gpulucas_gb300
    return gpulucas_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle
