"""Shared fixtures. Tests marked ``gpu`` need a GB300 and the built library;
everything else runs on the CPU (oracle, host logic, library loading)."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "ref_golden.npz"))


@pytest.fixture(scope="session")
def port():
    """This project's CPU restatement of the reference (the checker)."""
    from oracle import oracle

    if not oracle.available("port"):
        oracle.build_port()
    return oracle.Oracle("port")


@pytest.fixture(scope="session")
def lib():
    import mpsft_gb300 as m

    if not os.path.exists(m.LIB_PATH):
        from mpsft_gb300 import build

        build.build()
    return m.load_library()


@pytest.fixture(scope="session")
def ctx(lib):
    import mpsft_gb300 as m

    c = m.Context(0)
    yield c
    c.close()
