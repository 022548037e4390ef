"""Shared test fixtures.

Tests marked ``gpu`` need a CUDA device and the built native library; the
rest run on any host (the oracle, the golden fixtures, the host-side set-up
and the library's exported symbols).
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built library")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def oracle_built():
    """Build the oracle restatement (and the reference build, where its sources exist)."""
    from oracle import oracle
    oracle.build(ref=True)
    return oracle


@pytest.fixture(scope="session")
def native_lib():
    """The native library, built in-tree if needed."""
    from lulesh_gb300 import build
    build.build()
    import lulesh_gb300
    return lulesh_gb300.load()
