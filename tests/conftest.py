"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "magnetic-force_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    orc.build(ref=False)
    return orc.Oracle()


@pytest.fixture(scope="session")
def ref_kernels():
    import oracle as orc
    if not orc.RefKernels.available():
        pytest.skip("oracle/_ref (the reference's own kernels) is not built here")
    return orc.RefKernels()


@pytest.fixture(scope="session")
def mf():
    import build as mfbuild
    mfbuild.build()
    import mfgb
    mfgb.load()
    return mfgb


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
