"""mf_direct_field_noalloc: the direct field evaluation for callers that
cannot allocate device memory (their memory budget belongs to their own pool
allocator, or their loop cannot take cudaMalloc's synchronisation).

Called through the C ABI with ctypes and compared with mf_direct_field, the
allocating entry point, on two calls in a row (the second call reuses the
static scratch the first one left behind).  Kept in a file that sorts last so
a run stopping at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2, as for the other FP32 kernel tests


def _rel(a, b):
    return float(np.linalg.norm(a.astype(np.float64) - b.astype(np.float64)) / np.linalg.norm(b.astype(np.float64)))


def _noalloc_fn(mf):
    f = mf.load().mf_direct_field_noalloc
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                  ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_noalloc_matches_allocating_entry_point(mf, cuda):
    torch = cuda
    f = _noalloc_fn(mf)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(42)
    for n, h in ((5000, 0.03), (20000, 0.02)):  # two calls in a row, different sizes
        x = torch.from_numpy(rng.random((n, 3)).astype(np.float32)).cuda()
        m = torch.from_numpy(rng.normal(size=(n, 3)).astype(np.float32)).cuda()
        want = mf.direct_field(x, x, m, h).cpu().numpy()
        out = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
        st = f(ctypes.c_void_p(x.data_ptr()), n, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(m.data_ptr()), n,
               h, ctypes.c_void_p(out.data_ptr()), stream)
        assert st == 0, mf.load().mf_last_error()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert _rel(got, want) < TOL


def test_noalloc_rejects_oversize(mf, cuda):
    f = _noalloc_fn(mf)
    st = f(None, 65537, None, None, 10, 0.1, None, None)
    assert st == 1  # MF_ERR_INVALID_ARG
    assert b"65536" in mf.load().mf_last_error()
