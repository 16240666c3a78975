"""GPU tests of batched scenes (mf_batch_*): each scene's result in the batch
matches the same scene solved alone, and the FP64 oracle, within the FP32 bar
(relative L2 1e-5); graph-captured timesteps match uncaptured ones."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def mixed_scenes(seed=3, sizes=(301, 1001, 64, 2500, 777, 4096)):
    import scenes
    out = []
    for k, n in enumerate(sizes):
        rng = np.random.default_rng(seed + k)
        H = rng.normal(size=3)
        H /= np.linalg.norm(H)
        out.append(scenes.jittered_lattice(n, "sphere", radius=float(rng.uniform(0.2, 0.5)),
                                           chi=float(rng.uniform(0.5, 3.0)), seed=seed + k, H0=tuple(H)))
    return out


def test_batch_matches_single_scene_and_oracle(mf, oracle):
    scs = mixed_scenes()
    b = mf.Batch(scs)
    it, worst = b.solve(300, 1e-7)
    assert worst < 1e-7
    b.eval_force()
    for k, sc in enumerate(scs):
        s = mf.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos)
        s.set_option("solver", mf.SOLVER_CG)
        s.set_option("rel_tol", 1e-7)
        s.solve(300)
        s.evaluate_fitted_near_foece()
        assert rel(b.get(k, "total_B_over_mu0"), s.total_B_over_mu0) < 2e-6
        assert rel(b.get(k, "M"), s.M) < 2e-6
        assert rel(b.get(k, "magnetic_bodyforce"), s.magnetic_bodyforce) < 1e-5
        s.close()
    # one scene against the FP64 oracle
    sc = scs[2]
    hext, _ = oracle.ext(sc.pos, None, None, sc.H0, sc.h)
    bo, _, _ = oracle.solve_cg(sc.pos, sc.h, sc.c, hext, rel_tol=1e-13)
    assert rel(b.get(2, "total_B_over_mu0"), bo) < 1e-5
    assert rel(b.get(2, "magnetic_bodyforce"), oracle.force(sc.pos, sc.c * bo, sc.h)) < 1e-5


def test_alone_equals_in_the_mix(mf):
    scs = mixed_scenes(seed=11)
    mix = mf.Batch(scs)
    mix.solve(300, 1e-7)
    mix.eval_force()
    for k in (0, 3):
        alone = mf.Batch([scs[k]])
        alone.solve(300, 1e-7)
        alone.eval_force()
        assert rel(alone.get(0, "total_B_over_mu0"), mix.get(k, "total_B_over_mu0")) < 1e-6
        assert rel(alone.get(0, "magnetic_bodyforce"), mix.get(k, "magnetic_bodyforce")) < 1e-6
        alone.close()


def test_graph_steps_match_plain_steps(mf):
    scs = mixed_scenes(seed=21, sizes=(500, 1201, 333))
    a, g = mf.Batch(scs), mf.Batch(scs)
    for x in (a, g):
        x.solve(300, 1e-7)
    a.advance(1e-4, 5, iters_per_step=6, rel_tol=1e-7, graph=False)
    g.advance(1e-4, 5, iters_per_step=6, rel_tol=1e-7, graph=True)
    for k in range(3):
        for q in ("positions", "velocity", "total_B_over_mu0", "magnetic_bodyforce"):
            assert np.array_equal(a.get(k, q), g.get(k, q)), (k, q)


def test_counters_count_executed_pairs(mf):
    scs = mixed_scenes(seed=31, sizes=(400, 900))
    b = mf.Batch(scs)
    b.reset_counters()
    b.solve(300, 1e-7)
    rr, it = b.solver_state()
    c = b.counters()
    want = sum(sc.n ** 2 * (1 + i) for sc, i in zip(scs, it))
    assert c["field_pairs"] == pytest.approx(want)


CHILD = r"""
import sys
import numpy as np
sys.path[:0] = sys.argv[2:]
import mfgb
from test_gpu_batch import mixed_scenes
mfgb.load()
scs = mixed_scenes(seed=41, sizes=(4097, 6000, 9001))
b = mfgb.Batch(scs)
b.solve(300, 1e-7)
b.reset_counters()
b.eval_force()
out = {"launches": b.counters()["kernel_launches"]}
for k in range(len(scs)):
    out["F%d" % k] = b.get(k, "magnetic_bodyforce")
    out["B%d" % k] = b.get(k, "total_B_over_mu0")
a, g = mfgb.Batch(scs), mfgb.Batch(scs)
for x in (a, g):
    x.solve(300, 1e-7)
a.advance(1e-4, 3, iters_per_step=6, rel_tol=1e-7, graph=False)
g.advance(1e-4, 3, iters_per_step=6, rel_tol=1e-7, graph=True)
out["graph_equal"] = all(np.array_equal(a.get(k, q), g.get(k, q)) for k in range(len(scs))
                         for q in ("positions", "velocity", "magnetic_bodyforce"))
np.savez(sys.argv[1], **out)
"""


def test_packed_products_once_per_pair_in_batch(mf, tmp_path):
    # Scenes of the packed field and force paths in a child process with
    # MF_PAIR_SYMMETRIC=2 and MF_AUTOTUNE=0 (both read once per process): the
    # batch evaluates every field and force product once per unordered pair,
    # the CG's per-scene stop flags included -- a force product after a solve
    # is 6 launches: the marks of the scenes whose solve kept b (their force
    # comes from the solve's fused residual launch; none after this cold
    # solve), pair records, near-field correction, pair kernel, per-particle
    # finish, the force from the kept sums.  Each scene matches the same
    # scene solved alone, and graph-captured steps match plain steps bit for
    # bit.
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    pkg = os.path.join(os.path.dirname(here), "magnetic-force_gb300")
    path = str(tmp_path / "batch.npz")
    env = dict(os.environ, MF_AUTOTUNE="0", MF_PAIR_SYMMETRIC="2")
    subprocess.run([sys.executable, "-c", CHILD, path, here, pkg], env=env, check=True, timeout=600)
    got = np.load(path)
    assert int(got["launches"]) == 6
    assert bool(got["graph_equal"])
    for k, sc in enumerate(mixed_scenes(seed=41, sizes=(4097, 6000, 9001))):
        s = mf.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos)
        s.set_option("solver", mf.SOLVER_CG)
        s.set_option("rel_tol", 1e-7)
        s.solve(300)
        s.evaluate_fitted_near_foece()
        assert rel(got["B%d" % k], s.total_B_over_mu0) < 1e-5
        assert rel(got["F%d" % k], s.magnetic_bodyforce) < 1e-5
        s.close()
