"""Shared test set-up: import paths, the `gpu` marker, golden fixtures and library builds."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "jeju-stonewall-lbm_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libstonewall.so")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="session")
def native_lib():
    """libstonewall.so, built from csrc/ if it is missing or stale."""
    from stonewall import build, _native
    build.build()
    return _native.lib()


@pytest.fixture(scope="session")
def cuda(native_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but torch sees no CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.lib()
    return oracle
