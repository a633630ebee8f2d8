"""Test configuration: the ``gpu`` marker and import paths.

Tests marked ``gpu`` need a CUDA device and the built backend library; the
rest run on the CPU (oracle pins, host logic, ABI export checks).
"""
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
for p in (REPO, REPO / "pennylane-lightning_gb300", REPO / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built GB300 library")


@pytest.fixture(scope="session")
def oracle():
    from oracle.build_oracle import build_restatement
    from oracle.pyoracle import Oracle

    build_restatement()
    return Oracle("orc")


@pytest.fixture(scope="session")
def ops_module():
    import lightning_gb300.lightning_gb300_ops as ops

    return ops
