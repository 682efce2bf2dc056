"""Shared fixtures.  GPU tests are marked `gpu` and call the CUDA path
through the C ABI (libcwa.so); everything else runs on the CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def lib():
    """libcwa.so, built in-tree if missing."""
    from coupledwateranimation_gb300 import _abi, build
    if not _abi.LIB_PATH.exists():
        build.build()
    return _abi.load()


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure)."""
    from oracle import oracle
    oracle.build()
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def cuda_ok():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True
