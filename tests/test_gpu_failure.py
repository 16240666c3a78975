"""GPU tests of the bounded-wait error path, without a GPU fault.

Every staging wait in the pair kernels is bounded; when one runs out the CTA
records a device error word, waits (with the default bound) for the bulk
copies it has in flight, and leaves.  mf_debug_stage_wait_limit(0) makes the
staging waits give up at once, so every CTA takes that path: the call must
return MF_ERR_TIMEOUT, and the next call, with the default bound restored,
must return correct results (the scratch was reset).  The reference checks
nothing here (cuda_abstract_vector.cuh:169-175).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MF_ERR_TIMEOUT = 5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def timed_out(mf, fn):
    lib = mf.load()
    mf.check(lib.mf_debug_stage_wait_limit(0))
    try:
        with pytest.raises(mf.MFError) as e:
            fn()
        return e.value.status == MF_ERR_TIMEOUT
    finally:
        mf.check(lib.mf_debug_stage_wait_limit(-1))


def test_allpairs_wait_timeout_then_recovers(mf, oracle, cuda):
    # Separate targets and sources: the all-pairs kernel.
    torch = cuda
    rng = np.random.default_rng(61)
    tg = rng.uniform(-0.5, 0.5, (3000, 3)).astype(np.float32)
    src = rng.uniform(-0.5, 0.5, (5000, 3)).astype(np.float32)
    m = rng.normal(size=(5000, 3)).astype(np.float32)
    h = 0.04
    t, s, q = (torch.from_numpy(x).cuda() for x in (tg, src, m))
    assert timed_out(mf, lambda: mf.direct_field(t, s, q, h))
    want = oracle.field(tg.astype(np.float64), src.astype(np.float64), m.astype(np.float64), h)
    for _ in range(2):  # the next calls run with the default bound and are correct
        got = mf.direct_field(t, s, q, h).cpu().numpy()
        assert rel(got, want) < 1e-5


def test_once_per_pair_wait_timeout_then_recovers(mf, oracle, cuda):
    # One particle set of 40,000: the force once per unordered pair (k_sym).
    torch = cuda
    import scenes
    sc = scenes.jittered_lattice(40000, "sphere", radius=0.5, chi=2.0, seed=62)
    mom = ((np.array([0.0, 0.0, 1.0]) + 0.2 * np.random.default_rng(63).normal(size=(sc.n, 3))) * sc.c)
    p, q = torch.from_numpy(sc.pos).cuda(), torch.from_numpy(mom.astype(np.float32)).cuda()
    assert timed_out(mf, lambda: mf.direct_force(p, q, sc.h))
    got = mf.direct_force(p, q, sc.h).cpu().numpy()
    idx = np.sort(np.random.default_rng(64).choice(sc.n, 256, replace=False))
    p64 = sc.pos.astype(np.float64)
    T = oracle.tensor_sum(p64[idx], p64, mom, sc.h).reshape(-1, 3, 3)
    want = np.einsum("icr,ic->ir", T, mom[idx])
    assert rel(got[idx], want) < 1e-5


def test_solver_reports_timeout(mf):
    # A handle whose products time out reports MF_ERR_TIMEOUT from the solve;
    # a fresh handle afterwards solves normally.
    import scenes
    sc = scenes.jittered_lattice(20000, "sphere", radius=0.5, chi=2.0, seed=65)

    def make():
        s = mf.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos)
        s.set_option("solver", mf.SOLVER_CG)
        s.set_option("cg_max_iter", 5)
        return s

    s = make()
    assert timed_out(mf, lambda: s.solve(5))
    s.close()
    s = make()
    it, rr = s.solve(5)
    assert np.all(np.isfinite(s.total_B_over_mu0)) and rr < 1e-2
    s.close()
