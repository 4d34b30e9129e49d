"""Shared test set-up.

Tests marked ``gpu`` need a CUDA device and the built native library; they
are skipped when no device is present.  Every other test runs on the CPU.
"""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config: pytest.Config) -> None:
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def _cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_runtest_setup(item: pytest.Item) -> None:
    if item.get_closest_marker("gpu") is not None and not _cuda_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o

    o.build()
    return o


@pytest.fixture(scope="session")
def native():
    """The loaded native library (built if needed)."""
    from rlic_gb300 import _build, _native

    _build.build()  # incremental: recompiles only what changed
    return _native.lib()
