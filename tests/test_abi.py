"""CPU checks of the C ABI library: it loads, exports everything include/*.h
declares, and refuses politely without a GPU (no compute calls here)."""
import ctypes

import pytest


def test_exports_every_declared_symbol(mf):
    lib = mf.load()
    declared = mf.declared_symbols()
    assert len(declared) >= 25
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_strings(mf):
    lib = mf.load()
    assert lib.mf_abi_version() == 1
    assert lib.mf_status_string(0) == b"MF_OK"
    assert lib.mf_status_string(5) == b"MF_ERR_TIMEOUT"


def test_null_arguments_rejected(mf):
    lib = mf.load()
    assert lib.mf_create(None, None) == 1
    assert lib.mf_solve(None, 10, None, None) == 1
    assert lib.mf_destroy(None) == 0


def test_create_without_gpu(mf):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    g = np.zeros((2, 3), np.float32)
    g[1, 0] = 1
    with pytest.raises(mf.MFError) as e:
        mf.Solver(2, 1.0, 1.0, 1.0, 1.0, [0, 1, 0], None, None, g)
    assert e.value.status == 7  # MF_ERR_UNSUPPORTED
