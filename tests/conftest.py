import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libcrashcat_gpu.so")


def pytest_collection_modifyitems(config, items):
    import torch  # noqa: F401  (torch is only used to probe the device)
    has_gpu = torch.cuda.is_available()
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; fails loudly without it."""
    from crashcat_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as obuild, pyoracle
    obuild.build()
    return pyoracle.load()
