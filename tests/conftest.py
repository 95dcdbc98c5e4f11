"""pytest configuration: the ``gpu`` marker and shared fixtures.

CPU tests (``-m "not gpu"``) check the oracle against the golden fixtures made
from the reference, the host-side set-up and the C ABI's exports.  GPU tests
(``-m gpu``) compare the CUDA path, called through the C ABI, with the oracle.
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Build (if stale) the product library and the oracle before any test."""
    from fdtd_gb300 import build as fbuild
    from oracle import build as obuild

    fbuild.build()
    obuild.build_oracle()
    yield


@pytest.fixture(scope="session")
def golden() -> Path:
    return ROOT / "tests" / "golden"


@pytest.fixture(scope="session")
def cuda():
    """Skips unless a CUDA device is visible; returns torch."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
