"""mf_direct_field_noalloc: the direct field evaluation for callers that
cannot allocate device memory (their memory budget belongs to their own pool
allocator, or their loop cannot take cudaMalloc's synchronisation).

Called through the C ABI with ctypes, on two calls in a row (the second call
reuses the static scratch the first one left behind), and compared with
mf_direct_field, the allocating entry point, and with the FP64 oracle.  The
limits are covered too: 65,536 targets and sources (every ticket and every
partial-sum slot of the static array in use), target and source counts that
differ in both directions, no sources, and a call after a refused one.  Kept
in a file that sorts last so a run stopping at the first failure has run
every other test first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2, as for the other FP32 kernel tests


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) /
                 np.linalg.norm(np.asarray(b, np.float64)))


def _noalloc_fn(mf):
    f = mf.load().mf_direct_field_noalloc
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                  ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _call(mf, torch, t, s, m, h):
    f = _noalloc_fn(mf)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = torch.full((t.shape[0], 3), float("nan"), dtype=torch.float32, device="cuda")
    st = f(ctypes.c_void_p(t.data_ptr()), t.shape[0], ctypes.c_void_p(s.data_ptr()), ctypes.c_void_p(m.data_ptr()),
           s.shape[0], h, ctypes.c_void_p(out.data_ptr()), stream)
    assert st == 0, mf.load().mf_last_error()
    return out.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_and_oracle(mf, oracle, cuda):
    torch = cuda
    rng = np.random.default_rng(42)
    # two calls in a row: one particle set, then separate targets and sources
    cases = [(5000, 5000, 0.03, True), (3000, 7000, 0.02, False)]
    for nt, ns, h, same in cases:
        xs = rng.random((ns, 3)).astype(np.float32)
        xt = xs if same else rng.random((nt, 3)).astype(np.float32)
        m = rng.normal(size=(ns, 3)).astype(np.float32)
        t, s, q = (torch.from_numpy(a).cuda() for a in (xt, xs, m))
        if same:
            t = s
        got = _call(mf, torch, t, s, q, h)
        assert np.all(np.isfinite(got))
        want = mf.direct_field(t, s, q, h).cpu().numpy()
        assert _rel(got, want) < TOL
        ref = oracle.field(xt.astype(np.float64), xs.astype(np.float64), m.astype(np.float64), h)
        assert _rel(got, ref) < TOL


def test_noalloc_limits(mf, oracle, cuda):
    torch = cuda
    rng = np.random.default_rng(43)
    n = 65536
    x = rng.random((n, 3)).astype(np.float32)
    m = rng.normal(size=(n, 3)).astype(np.float32)
    h = 0.01
    X, M = torch.from_numpy(x).cuda(), torch.from_numpy(m).cuda()
    x64, m64 = x.astype(np.float64), m.astype(np.float64)
    # 65,536 x 65,536: every target block's ticket and the full grid of partials
    got = _call(mf, torch, X, X, M, h)
    idx = np.sort(rng.choice(n, 512, replace=False))
    assert _rel(got[idx], oracle.field(x64[idx], x64, m64, h)) < TOL
    # 65,536 targets x 3 sources, and 1 target x 65,536 sources
    got = _call(mf, torch, X, X[:3].contiguous(), M[:3].contiguous(), h)
    assert _rel(got[idx], oracle.field(x64[idx], x64[:3], m64[:3], h)) < TOL
    got = _call(mf, torch, X[7:8].contiguous(), X, M, h)
    assert _rel(got, oracle.field(x64[7:8], x64, m64, h)) < TOL
    # no sources: zeros
    f = _noalloc_fn(mf)
    out = torch.full((10, 3), float("nan"), dtype=torch.float32, device="cuda")
    st = f(ctypes.c_void_p(X.data_ptr()), 10, None, None, 0, h, ctypes.c_void_p(out.data_ptr()),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0 and np.all(out.cpu().numpy() == 0.0)
    # beyond the limit: refused with a clear error; the next call works
    st = f(None, 65537, None, None, 10, 0.1, None, None)
    assert st == 1  # MF_ERR_INVALID_ARG
    assert b"65536" in mf.load().mf_last_error()
    st = f(ctypes.c_void_p(X.data_ptr()), 10, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(M.data_ptr()), 65537,
           h, ctypes.c_void_p(out.data_ptr()), None)
    assert st == 1
    got = _call(mf, torch, X[:2000].contiguous(), X, M, h)
    assert _rel(got, oracle.field(x64[:2000], x64, m64, h)) < TOL
