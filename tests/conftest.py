"""Shared pytest setup: the `gpu` marker, import paths and common fixtures."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def golden() -> dict:
    return json.loads((GOLDEN / "reference_golden.json").read_text())


@pytest.fixture(scope="session")
def qlib():
    """The product library (loads without a GPU; only host-side calls are made on CPU)."""
    import quasi_gb300
    from quasi_gb300 import build as qbuild

    qbuild.build()
    return quasi_gb300.load_library()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as o

    o.build()
    return o


@pytest.fixture(scope="session")
def cuda_ok():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return True
