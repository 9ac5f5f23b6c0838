import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Build the native libraries once per session (no-op when up to date)."""
    import __graft_entry__

    __graft_entry__._build_module().build()
    return True


@pytest.fixture(scope="session")
def ffrs_gpu(built):
    import libffrs_gb300

    return libffrs_gb300.libffrs


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))
