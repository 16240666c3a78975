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
    discard the kept sums too;
  * in a batch, scenes whose solve kept b take the force from the kept sums
    and the others their own force product, in the same step.
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


# A batch whose packed scenes run both products once per unordered pair
# (MF_PAIR_SYMMETRIC=2 in a child process: the mode is read once per
# process), with and without the fused residual launch (MF_FUSED_PRODUCTS).
_BATCH_CHILD = r"""
import sys
import numpy as np
sys.path[:0] = sys.argv[2].split(":")
import mfgb, scenes
scs = []
for k, n in enumerate((6000, 2500, 9001, 512, 4096)):
    rng = np.random.default_rng(40 + k)
    H = rng.normal(size=3); H /= np.linalg.norm(H)
    scs.append(scenes.jittered_lattice(n, "sphere", radius=float(rng.uniform(0.3, 0.5)),
                                       chi=float(rng.uniform(0.5, 3.0)), seed=40 + k, H0=tuple(H)))
K = len(scs)
get = lambda b, q: [b.get(k, q) for k in range(K)]
b = mfgb.Batch(scs)
out = {"h": np.array([sc.h for sc in scs]), "pos0": get(b, "positions")}
b.solve(300, 1e-3)                     # a loose cold solve: every scene iterates
b.eval_force()
out["F_cold"], out["M_cold"] = get(b, "magnetic_bodyforce"), get(b, "M")
b.solve(0, 1.0)                        # no iteration: each scene's residual of its b
rr, _ = b.solver_state()
tol = float(np.median(rr[[0, 2, 4]]))  # packed force scenes below it keep b, the others iterate
b.solve(300, tol)
_, out["iters_mixed"] = b.solver_state()
b.eval_force()
out["F_mixed"], out["M_mixed"] = get(b, "magnetic_bodyforce"), get(b, "M")
b.solve(300, 1e-6)
b.advance(1e-4, 3, 4, 1e-6, True)      # warm steps: every scene keeps b
_, out["iters_warm"] = b.solver_state()
out["F_warm"], out["M_warm"], out["pos_warm"] = get(b, "magnetic_bodyforce"), get(b, "M"), get(b, "positions")
out["launches"] = b.counters()["kernel_launches"]
np.savez(sys.argv[1], **{k: np.array(v, dtype=object) if isinstance(v, list) else v for k, v in out.items()})
"""


def _run_batch_child(tmp_path, fused):
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, MF_PAIR_SYMMETRIC="2", MF_AUTOTUNE="0", MF_FUSED_PRODUCTS=str(fused))
    out = os.path.join(str(tmp_path), f"batch{fused}.npz")
    path = ":".join([os.path.join(root, "magnetic-force_gb300"), root])
    r = subprocess.run([sys.executable, "-c", _BATCH_CHILD, out, path], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    z = np.load(out, allow_pickle=True)
    return {k: z[k] for k in z.files}


def test_batch_fused_matches_separate_products(mf, oracle, tmp_path):
    a = _run_batch_child(tmp_path, 1)
    b = _run_batch_child(tmp_path, 0)
    assert a["launches"] > b["launches"]  # the kept-scene marking and the force from kept sums
    packed = (0, 2, 4)  # the scenes of >= 4,096 particles: packed force, once per unordered pair

    def force_ok(z, F, M, pos):
        for k in packed:
            want = oracle.force(np.asarray(z[pos][k], np.float64), np.asarray(z[M][k], np.float64),
                                float(z["h"][k]), None)
            assert rel(z[F][k], want) < 1e-5, (F, k)

    # Cold solve (every scene iterates): the force products.
    force_ok(a, "F_cold", "M_cold", "pos0")
    # A mixed solve: one packed scene keeps its b (force from the kept sums),
    # the others iterate from a b 1e-3 off (their kept sums are stale by that
    # much, so taking them would miss the oracle by ~1e-3).
    its = a["iters_mixed"]
    assert (its[list(packed)] == 0).any() and (its[list(packed)] > 0).any(), its
    force_ok(a, "F_mixed", "M_mixed", "pos0")
    # Warm steps: every scene keeps b.  Against the separate products: both
    # solved to 1e-6 relative residual first (a different iteration count at
    # that bar moves b by a few 1e-6).
    assert (a["iters_warm"] == 0).all()
    force_ok(a, "F_warm", "M_warm", "pos_warm")
    for k in range(5):
        assert rel(a["F_warm"][k], b["F_warm"][k]) < 1e-5
        assert rel(a["M_warm"][k], b["M_warm"][k]) < 1e-5
