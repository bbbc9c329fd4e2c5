"""Test configuration: the `gpu` marker, the package loader and the oracle."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def ora():
    from oracle import build as oracle_build
    from oracle import ora as oracle_mod

    oracle_build.build()
    return oracle_mod


@pytest.fixture(scope="session")
def fg():
    """The library package (fhe.rs_gb300/ imported as `fhe_gb300`), built."""
    import __graft_entry__ as ge

    mod = ge.load_package()
    mod.build()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def cuda(fg):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu tests")
    torch.cuda.set_device(0)
    return torch
