import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsdfibm_cuda.so")
    config.addinivalue_line("markers", "first_gpu_run: a GPU test that has not yet run on a GPU (ordered last)")


def pytest_collection_modifyitems(config, items):
    # tests that have not yet run on a GPU go last, so that under -x a failure there hides no other result
    items.sort(key=lambda it: it.get_closest_marker("first_gpu_run") is not None)


@pytest.fixture(scope="session")
def cuda_lib():
    """The in-tree CUDA library, built on first use when missing (nvcc cross-compiles without a GPU)."""
    from sdfibm_gb300 import build
    build.build()
    from sdfibm_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def golden(name):
    return np.load(os.path.join(ROOT, "tests", "golden", name))
