import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsu2g.so")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (C restatement of the reference), built on demand."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as o

    o.build()
    return o


@pytest.fixture(scope="session")
def su2lib():
    """libsu2g.so, built on demand (host entry points work without a GPU)."""
    from su2dmrg_gb300 import _build, capi

    _build.build()
    return capi.lib()


GOLDEN = os.path.join(REPO, "tests", "golden")
