import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libbandedgpu.so")


@pytest.fixture(scope="session")
def bm():
    """The host package (bandedmatrices.jl_gb300), with the CUDA library loaded."""
    import __graft_entry__ as ge

    pkg = ge.package()
    return pkg


@pytest.fixture(scope="session")
def gpu(bm):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    bm.load_library()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.lib()
    return oracle
