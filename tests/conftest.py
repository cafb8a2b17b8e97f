"""Test configuration: the ``gpu`` marker, and build steps for the oracle
(test infrastructure) and the CUDA library (cross-compiled for sm_103a)."""

from __future__ import annotations

import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; built if missing.  GPU tests fail if it cannot load."""
    from titsolver_gb300 import _abi, build

    build.build()
    return _abi.load()
