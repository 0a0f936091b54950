"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cuda-pbf-fluid-sim_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI of libpbf_gb300)")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__ as g

    g.build_library()
    g.build_oracle()
    return True


@pytest.fixture(scope="session")
def lib(built):
    import pbfx

    return pbfx.load()


@pytest.fixture(scope="session")
def orc(built):
    import pbfx

    return pbfx.load_oracle()


def cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(lib):
    if not cuda_available():
        pytest.fail("test marked gpu but no CUDA device is visible")
    import torch

    torch.cuda.init()
    return torch
