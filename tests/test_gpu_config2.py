"""GPU tests at the headline scene's full size: 65,536 particles in a
jittered-lattice sphere (h = 2 spacings, chi = 2, H0 = (0, 0, 1)), solved and
compared over ALL particles with the FP64 oracle's own solution
(tests/golden/config2_oracle.npz: oracle CG to a relative residual of 6e-12,
then the oracle's Kelvin force at M = c b).

Bars, relative L2 over all particles and components:
  B/mu0, M, Kelvin force   1e-5   (all-pairs path and FMM path alike)
The solve stops at the bench's tolerance (relative residual 1e-6); the
system is well conditioned, so B and M land within a few 1e-6 of the
oracle's solution.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), "golden", "config2_oracle.npz")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def config2():
    z = np.load(FIX)
    return {k: z[k] for k in z.files}


def solved(mf, z, rel_tol, **opts):
    n = len(z["pos"])
    s = mf.Solver(n, float(z["h"]), float(z["h"]), float(z["volume"]), float(z["chi"]), z["H0"], None, None,
                  z["pos"], precision="fp32")
    s.set_option("solver", mf.SOLVER_CG)
    s.set_option("rel_tol", rel_tol)
    for k, v in opts.items():
        s.set_option(k, v)
    it, rr = s.solve(500)
    assert rr < rel_tol
    s.evaluate_fitted_near_foece()
    return s


@pytest.mark.parametrize("rel_tol", [1e-6, 1e-8])
def test_allpairs_solution_matches_oracle(mf, config2, rel_tol):
    z = config2
    c = float(z["volume"]) * float(z["chi"]) / (1.0 + float(z["chi"]))
    s = solved(mf, z, rel_tol)
    assert s.fmm_stats()["active"] == 0
    eb = rel(s.total_B_over_mu0, z["b"])
    em = rel(s.M, c * z["b"].astype(np.float64))
    ef = rel(s.magnetic_bodyforce, z["F"])
    assert eb < 1e-5 and em < 1e-5 and ef < 1e-5, (eb, em, ef)
    s.close()


def test_fmm_solution_matches_oracle(mf, config2):
    # Both products through the FMM at the defaults (P = 8; field aperture
    # 0.5, force aperture 0.44, P = 10) on the same scene.
    z = config2
    c = float(z["volume"]) * float(z["chi"]) / (1.0 + float(z["chi"]))
    s = solved(mf, z, 1e-7, fmm=mf.FMM_ON)
    st = s.fmm_stats()
    assert st["active"] == 1 and st["force_active"] == 1 and st["degree"] == 7
    assert st["theta"] == 0.5 and abs(st["force_theta"] - 0.44) < 1e-12
    # the force's own, wider near lists (equal where the leaf boxes make them so)
    assert st["force_p2p_pairs"] >= st["p2p_pairs"] and s.get_option("fmm_force_order") == 10
    eb = rel(s.total_B_over_mu0, z["b"])
    em = rel(s.M, c * z["b"].astype(np.float64))
    ef = rel(s.magnetic_bodyforce, z["F"])
    assert eb < 1e-5 and em < 1e-5 and ef < 1e-5, (eb, em, ef)
    s.close()


def test_fused_step_matches_oracle(mf, config2):
    # Warm steps at the full size: once the warm start stands, the solve's
    # residual and the Kelvin force come from one launch (field and force
    # once per unordered pair); the state and force still match the oracle.
    z = config2
    c = float(z["volume"]) * float(z["chi"]) / (1.0 + float(z["chi"]))
    s = solved(mf, z, 1e-6)
    f_sep = s.magnetic_bodyforce.copy()
    s.set_option("kernel_timing", 1)
    for _ in range(2):
        it, rr = s.solve(500)
        assert it == 0 and rr < 1e-6
    s.evaluate_fitted_near_foece()
    assert s.kernel_stats("field_force")["launches"] == 1 and s.kernel_stats("force")["launches"] == 0
    ef = rel(s.magnetic_bodyforce, z["F"])
    assert rel(s.magnetic_bodyforce, f_sep) < 2e-6
    eb = rel(s.total_B_over_mu0, z["b"])
    em = rel(s.M, c * z["b"].astype(np.float64))
    assert eb < 1e-5 and em < 1e-5 and ef < 1e-5, (eb, em, ef)
    s.close()
