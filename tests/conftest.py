"""Shared pytest configuration.

Markers:
  gpu  -- needs a CUDA GPU (runs the libvgnav kernels); deselect with -m "not gpu".
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU and the libvgnav kernels")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def vgnav():
    """The product library, built in-tree (nvcc) if needed."""
    from vecgeom_gb300 import build

    build.build()
    import vecgeom_gb300

    return vecgeom_gb300


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required for tests marked gpu")
    return torch
