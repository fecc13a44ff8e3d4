import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pbd-simulation-framework-cuda_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    # keep collection order but make sure the no-allocation test file runs last
    items.sort(key=lambda it: 1 if "test_zz_" in it.nodeid else 0)


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def pbd():
    import pbd as m
    return m


@pytest.fixture(scope="session")
def scenes():
    import scenes as m
    return m


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as m
    return m


@pytest.fixture(scope="session")
def need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def small_params(pbd, scenes, box=16, rho0=1000.0, eps=0.1, vorticity=0.0, viscosity=0.0, iterations=4):
    p = scenes.workload_params(pbd, box, rho0, vorticity=vorticity, viscosity=viscosity, iterations=iterations)
    p.lambda_epsilon = eps
    return p
