"""Shared test setup.

Marker `gpu`: needs a CUDA GPU (run with -m gpu on the GB300); everything else
runs on CPU. The library is built in-tree on first use (nvcc cross-compiles
without a GPU), so a fresh checkout needs no separate build step.
"""

from __future__ import annotations

import importlib
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

PKG_NAME = "21cma_abf_correlator_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def package():
    return importlib.import_module(PKG_NAME)


def built_library():
    build = importlib.import_module(PKG_NAME + ".build")
    return build.build()


@pytest.fixture(scope="session")
def pkg():
    built_library()
    return package()


@pytest.fixture(scope="session")
def lib(pkg):
    return pkg.abi.load()


@pytest.fixture(scope="session")
def oracle():
    return importlib.import_module("oracle.corr_oracle")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
