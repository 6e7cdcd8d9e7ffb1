"""Shared fixtures. Tests marked ``gpu`` need a CUDA device (run on the GB300);
everything else runs on the CPU."""
import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, build
    build()
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    data = np.load(os.path.join(GOLDEN, "golden.npz"))
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    return data, meta


@pytest.fixture(scope="session")
def golden_cases():
    sys.path.insert(0, GOLDEN)
    import make_golden
    return make_golden.cases()


@pytest.fixture(scope="session")
def solver_lib():
    """The CUDA library (built in-tree when missing)."""
    from sparsesolv_gb300 import _native
    if not os.path.exists(_native.SOLVER_LIB):
        _native.build_solver()
    return _native.load_solver()


@pytest.fixture(scope="session")
def gpu(solver_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    return solver_lib
