"""Test configuration: the `gpu` marker and import paths.

CPU tests (-m "not gpu") cover the oracle, the golden fixtures, host logic
and that libkdgb.so loads and exports its ABI.  GPU tests (-m gpu) run the
CUDA path through the C ABI and compare it with the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "extensions-photonmapping_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def kdgb_lib():
    """The built CUDA library (built in-tree on first use)."""
    import kdgb
    from kdgb import _build
    _build.build()
    return kdgb


@pytest.fixture(scope="session")
def cuda(kdgb_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test without a CUDA device")
    return torch
