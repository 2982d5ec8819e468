"""pytest configuration: the `gpu` marker and shared fixtures.

`-m gpu` tests call the CUDA library through its C-ABI and compare against the
CPU oracle; `-m "not gpu"` tests run on any host (oracle KATs, host logic,
library symbol table).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU on this host")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def gpulib():
    """Build (if needed) and load the CUDA library; fail loudly if it cannot load."""
    from aeros_gb300 import build as b
    b.build()
    from aeros_gb300 import _capi
    return _capi.lib()
