"""Test configuration: the `gpu` marker, import paths, and the builds the tests need.

`-m "not gpu"` runs everywhere (the oracle against the reference's pins and golden vectors, the C
ABI's exports and layouts, the host logic, the multi-process plumbing on gloo); `-m gpu` runs the
CUDA path against the oracle on a GB300.
"""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.join(ROOT, "tests")
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (a GB300) and libwlcuda.so")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def wl_lib():
    """libwlcuda.so, built in-tree if it is missing (nvcc cross-compiles without a GPU)."""
    import game_engine_gb300 as g
    if not os.path.exists(g.LIB_PATH):
        g.build()
    return g.lib()


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(wl_lib, oracle_mod):
    """The CUDA path: the library and a device. A GPU test fails loudly without one."""
    if not cuda_available():
        pytest.fail("no CUDA device: the gpu tests run on a GB300")
    return wl_lib
