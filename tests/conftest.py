"""Shared fixtures.  Tests marked ``gpu`` need a GB300 and the built library;
everything else runs on any CPU host (``pytest -m "not gpu"``)."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure), built on first use."""
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, "golden_arrays.npz")))
    return meta, arrays


@pytest.fixture(scope="session")
def built_lib():
    """Path of libginf_gb300.so, compiled in tree if needed."""
    import gridinfcuda_gb300
    return gridinfcuda_gb300.build()


@pytest.fixture(scope="session")
def ginf(built_lib):
    """The C-ABI binding on a GPU host; fails (never skips) without a GPU."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from gridinfcuda_gb300 import capi
    capi.lib()
    return capi
