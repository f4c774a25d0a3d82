"""Shared fixtures. Tests marked `gpu` need a GB300 and the built library;
everything else runs on the CPU (the oracle, host logic, ABI exports)."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def oracle():
    from oracle.bind import Oracle

    return Oracle()


@pytest.fixture(scope="session")
def reference_available():
    from oracle.bind import Reference, build_reference

    if not Reference.available():
        try:
            build_reference()
        except Exception:
            pass
    return Reference.available()


@pytest.fixture(scope="session")
def native():
    """The CUDA library. Fails (never skips) when it is missing."""
    from computer_graphics_lab_00_gb300 import abi

    return abi.load()
