import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")
    # The checker (oracle) and the product library are built in-tree; both
    # builds are idempotent and quick when nothing changed.
    from oracle import build_oracle

    build_oracle.build_oracle()
    build_oracle.build_ref()
    from sycldb_gb300 import build

    build.build()


def gpu_available() -> bool:
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


@pytest.fixture(autouse=True)
def _release_device_buffers(request):
    yield
    if "gpu" in request.keywords:
        from tests import gpu_util

        gpu_util.release()
