"""Shared pytest configuration: the ``gpu`` marker and import paths."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import prism_oracle

    prism_oracle.build_oracle()
    return prism_oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The native library on a GPU machine; fails (never skips) when it is missing."""
    import torch

    from harmonica_gb300 import _native

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    _native.build()
    return _native.lib()
