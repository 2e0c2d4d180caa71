"""Test configuration: the `gpu` marker and session-wide library builds.

CPU tests (`-m "not gpu"`) check the oracle against golden vectors, the host
logic and that the C-ABI library loads and exports every declared symbol.
GPU tests (`-m gpu`) are the parity tests proper; they call the solver
through the C ABI and compare with the oracle on the same seeded inputs.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    from tests import _oracle
    return _oracle


@pytest.fixture(scope="session")
def kamsta():
    from kamsta_gb300 import build
    build.build()
    import kamsta_gb300
    return kamsta_gb300
