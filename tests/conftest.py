"""Shared fixtures.

GPU tests (marked ``gpu``) call the CUDA library through its C ABI; the CPU
oracle under oracle/ is the checker. CPU tests never run device code.
"""
from __future__ import annotations

import importlib
import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
if str(ROOT / "oracle") not in sys.path:
    sys.path.insert(0, str(ROOT / "oracle"))

PACKAGE = "quantum-harness-peps-naive_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the device library through the C ABI)")


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "reference_golden.json").read_text())


@pytest.fixture(scope="session")
def oracle():
    import oracle_py

    oracle_py.build()
    return oracle_py


@pytest.fixture(scope="session")
def qp():
    mod = importlib.import_module(PACKAGE)
    if not mod.LIBRARY_PATH.exists():
        mod.build()
    return mod


@pytest.fixture(scope="session")
def ctx(qp):
    c = qp.Context(0)
    yield c
    c.close()
