"""GPU tests of the field and force evaluated in one launch (MF_OPT_FUSED_PRODUCTS).

A solve whose warm start stands leaves the magnetization unchanged, so the
Kelvin force asked for next is the force of the dipoles the solve's first
residual product already swept.  The handle then forms both in one launch
and the force comes from the kept pair sums.  Checked here:
  * the force from the fused launch equals the separate force product to
    FP32 rounding (2e-6) and the FP64 oracle's force of the same M (1e-5);
  * a fused launch whose solve then iterates is discarded: the force comes
    from the separate product;
  * new positions or an option change between the solve and the force
    discard the kept sums too.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 16385  # odd: a partial last block and a pair item without its partner


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def scene():
    import scenes
    return scenes.jittered_lattice(N, "sphere", radius=0.5, chi=2.0, seed=11)


def handle(mf, sc, fused):
    s = mf.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos, precision="fp32")
    s.set_option("solver", mf.SOLVER_CG)
    s.set_option("autotune", 0)
    s.set_option("pair_symmetric", 2)  # both products once per unordered pair at this size
    s.set_option("fused_products", fused)
    s.set_option("kernel_timing", 1)
    return s


def launches(s, kind):
    return s.kernel_stats(kind)["launches"]


def test_fused_force_matches_separate_product_and_oracle(mf, oracle, scene):
    sc = scene
    a, b = handle(mf, sc, 1), handle(mf, sc, 0)
    for s in (a, b):
        it, rr = s.solve(500)
        assert it > 0 and rr < 1e-6  # cold start: the solve iterates
        s.evaluate_fitted_near_foece()
        s.reset_counters()
        # the first warm solve finds its warm start standing; the second is
        # then evaluated together with the force
        for _ in range(2):
            it, rr = s.solve(500)
            assert it == 0 and rr < 1e-6
        s.evaluate_fitted_near_foece()
    assert launches(a, "field_force") == 1 and launches(a, "force") == 0 and launches(a, "field") == 1
    assert launches(b, "field_force") == 0 and launches(b, "force") == 1 and launches(b, "field") == 2
    assert a.counters()["force_pairs"] == b.counters()["force_pairs"] == float(N) * N
    # both cold solves ran the separate products: the same b
    assert rel(a.total_B_over_mu0, b.total_B_over_mu0) == 0.0
    fa, fb = a.magnetic_bodyforce, b.magnetic_bodyforce
    assert rel(fa, fb) < 2e-6
    want = oracle.force(sc.pos.astype(np.float64), a.M.astype(np.float64), sc.h, None)
    assert rel(fa, want) < 1e-5
    assert rel(fb, want) < 1e-5
    a.close()
    b.close()


def test_fused_launch_discarded_when_the_solve_iterates(mf, oracle, scene):
    sc = scene
    a, b = handle(mf, sc, 2), handle(mf, sc, 0)  # a: every solve's first residual is fused
    for s in (a, b):
        it, rr = s.solve(500)
        assert it > 0 and rr < 1e-6
        s.evaluate_fitted_near_foece()
    assert launches(a, "field_force") == 1 and launches(a, "force") == 1
    assert rel(a.total_B_over_mu0, b.total_B_over_mu0) < 1e-6
    assert rel(a.magnetic_bodyforce, b.magnetic_bodyforce) < 2e-6
    want = oracle.force(sc.pos.astype(np.float64), a.M.astype(np.float64), sc.h, None)
    assert rel(a.magnetic_bodyforce, want) < 1e-5

    # New positions between the solve and the force: the kept sums are stale.
    a.reset_counters()
    it, _ = a.solve(500)
    assert it == 0 and launches(a, "field_force") == 1
    a.setTargetpos(sc.pos)
    a.evaluate_fitted_near_foece()
    assert launches(a, "force") == 1
    assert rel(a.magnetic_bodyforce, want) < 1e-5

    # An option change likewise.
    a.reset_counters()
    it, _ = a.solve(500)
    assert it == 0 and launches(a, "field_force") == 1
    a.set_option("tolerance", 0.1)
    a.evaluate_fitted_near_foece()
    assert launches(a, "force") == 1
    assert rel(a.magnetic_bodyforce, want) < 1e-5

    with pytest.raises(mf.MFError):
        a.set_option("fused_products", 3)
    assert a.get_option("fused_products") == 2
    a.close()
    b.close()
