"""Shared pytest configuration: the `gpu` marker, import paths and build fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "hermite-teno_gb300"
for p in (str(PKG), str(REPO / "oracle"), str(REPO)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc  # oracle/oracle.py

    orc.lib()
    return orc


@pytest.fixture(scope="session")
def hteno_lib():
    """The CUDA library, built in-tree for sm_103a if it is missing or stale."""
    from hteno import build

    build.build_library()
    import hteno

    return hteno


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
