"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the native
library; everything else runs on the CPU (oracle, golden vectors, C-ABI
symbol and argument checks, host logic, gloo multi-process tests)."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the native library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def golden():
    return np.load(ROOT / "tests" / "golden" / "fft_golden.npz")


@pytest.fixture(scope="session")
def native():
    """The native library, built in-tree if it is not there yet."""
    import glscv_gb300
    if not glscv_gb300.LIB_PATH.exists():
        from glscv_gb300 import build
        build.build()
    return glscv_gb300.lib()


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu-marked tests")
    return torch


@pytest.fixture(scope="session")
def ctx(native, torch_cuda):
    import glscv_gb300
    c = glscv_gb300.Context(0)
    yield c
    c.close()
