import ast
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_hotpath.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN, allow_pickle=False)


def settings_of(golden, key):
    return ast.literal_eval(str(golden[key]))


@pytest.fixture(scope="session")
def oracle_port():
    from oracle import port
    port.build()
    return port


@pytest.fixture(scope="session")
def psim():
    import proteinsim2015_gb300 as psim
    psim.lib()
    return psim


@pytest.fixture(params=["rows", "cells"])
def force_pass(request, monkeypatch):
    """Both force-pass layouts: a warp per 32 sorted particles, a block per cell."""
    monkeypatch.setenv("PSIM_FORCE_PASS", request.param)
    return request.param
