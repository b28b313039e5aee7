"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import importlib
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


def pkg():
    return importlib.import_module("unnatural-planets_gb300")


def abi():
    return importlib.import_module("unnatural-planets_gb300.abi")


def workloads():
    return importlib.import_module("unnatural-planets_gb300.workloads")


@pytest.fixture(scope="session")
def up():
    return pkg()


@pytest.fixture(scope="session")
def W():
    return workloads()


@pytest.fixture(scope="session")
def O():
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test needs CUDA (run with -m 'not gpu' on a CPU-only machine)")
    pkg().load(build_if_missing=True)
    return torch


def rng(seed=0):
    return np.random.default_rng(seed)
