"""Shared test set-up: import paths, the `gpu` marker, and builds of the
library under test and of the oracle (the checker)."""
import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "cloning-lbm-mpi_gb300"
for p in (REPO, PKG, REPO / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def clbm_lib():
    import build as clbm_build
    clbm_build.build_library()
    import clbm
    return clbm


@pytest.fixture(scope="session")
def gpu(clbm_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
