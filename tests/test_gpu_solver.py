"""GPU parity of the solver object (the reference's cuda_magnet_cgOptimizer
surface) against the oracle: magnetization M, field B/mu0 and Kelvin force F.

Tolerances, relative L2 over all particles and components:
  FP32 solver vs FP64 oracle     1e-5
  FP64 solver vs FP64 oracle     1e-8
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def oracle_step(oracle, pos, h, volume, chi, H0, ext_pos=None, ext_m=None, ext_h=None, naive=False):
    """Converged FP64 solution and force for one scene."""
    pos = np.asarray(pos, np.float64)
    hs = h if naive else ext_h
    hext, rext = oracle.ext(pos, ext_pos, ext_m, H0, hs if hs else h)
    c = volume * chi / (1 + chi)
    b, it, rr = oracle.solve_cg(pos, h, c, hext, rel_tol=1e-13, max_iter=2000)
    M = c * b
    F = oracle.force(pos, M, h, rext if ext_pos is not None and len(ext_pos) else None, naive_quirks=naive)
    return dict(b=b, M=M, F=F, hext=hext, rext=rext)


def make(mf, sc, precision="fp32", ext_pos=None, ext_m=None, ext_h=None):
    return mf.Solver(sc.n, sc.h, ext_h if ext_h else sc.h, sc.volume, sc.chi, sc.H0, ext_pos, ext_m, sc.pos,
                     precision=precision)


@pytest.mark.parametrize("n", [8, 512, 3000])
def test_cg_fp32_matches_oracle(mf, oracle, n):
    import scenes
    sc = scenes.jittered_lattice(n, "sphere", radius=0.5, chi=2.0, seed=n)
    want = oracle_step(oracle, sc.pos, sc.h, sc.volume, sc.chi, sc.H0)
    s = make(mf, sc)
    s.set_option("solver", mf.SOLVER_CG)
    it, relres = s.solve(200)
    assert relres < 1e-6
    s.evaluate_fitted_near_foece()
    assert rel(s.total_B_over_mu0, want["b"]) < 1e-5
    assert rel(s.M, want["M"]) < 1e-5
    assert rel(s.magnetic_bodyforce, want["F"]) < 1e-5
    assert rel(s.Hext, want["hext"]) < 1e-7


def test_cg_fp64_plain_config(mf, oracle):
    # N=4096 uniform cube, V=(1/16)^3, h=0.125, chi=1, H0=(0,0,1), FP64 to 1e-8
    import scenes
    sc = scenes.config_plain_fp64()
    want = oracle_step(oracle, sc.pos, sc.h, sc.volume, sc.chi, sc.H0)
    s = make(mf, sc, "fp64")
    s.set_option("solver", mf.SOLVER_CG)
    s.set_option("rel_tol", 1e-10)
    it, relres = s.solve(500)
    assert relres < 1e-10
    s.evaluate_fitted_near_foece()
    assert rel(s.get("total_B_over_mu0", f64=True), want["b"]) < 1e-8
    assert rel(s.get("M", f64=True), want["M"]) < 1e-8
    assert rel(s.get("magnetic_bodyforce", f64=True), want["F"]) < 1e-8


def main_cu_scene():
    g = np.array([[i, j, k] for i in range(2) for j in range(2) for k in range(2)], np.float32)
    return g


def test_nlcg_reference_defaults_main_cu(mf, oracle):
    # magnetic_solver/main.cu: solve(100) with the reference's defaults
    # (tolerance 0.1 absolute RMS, max_iteration 80), then the force.
    g = main_cu_scene()
    ext_p = np.float32([[0, 0, 0]])
    ext_m = np.float32([[0, 1, 0]])
    s = mf.Solver(8, 1.0, 1.0, 1.0, 1.0, [0, 1, 0], ext_p, ext_m, g)
    assert s.tolerance == pytest.approx(0.1) and s.max_iteration == 80 and not s.naive
    it, err = s.solve(100)
    hext, rext = oracle.ext(g, ext_p, ext_m, [0, 1, 0], 1.0)
    b_o, errs_o, steps_o = oracle.solve_nlcg(g, 1.0, 1.0, 1.0, hext, tolerance=0.1, niter=100, max_iteration=80)
    hist = s.error_history()
    assert it == steps_o
    assert len(hist) == len(errs_o)
    assert rel(hist, errs_o) < 1e-5
    assert rel(s.total_B_over_mu0, b_o) < 1e-5
    s.evaluate_fitted_near_foece()
    F_o = oracle.force(g, 0.5 * b_o, 1.0, rext)
    assert rel(s.magnetic_bodyforce, F_o) < 1e-5
    assert rel(s.dHextdx, rext[:, 0:3]) < 1e-5
    assert rel(s.dHextdz, rext[:, 6:9]) < 1e-5
    # main.cu:48 moves the targets (7 of them remain after the update) and re-solves
    upd = np.float32([[i, j, k + 1] for i in range(2) for j in range(2) for k in range(1)])
    s.setTargetpos(upd)
    s.setHext([0, 1, 0], ext_p, ext_m, 1.0)
    s.solve(100)
    s.evaluate_fitted_near_foece()
    assert s.np == 4
    assert np.all(np.isfinite(s.magnetic_bodyforce))


def test_nlcg_tight_matches_cg(mf, oracle):
    import scenes
    sc = scenes.jittered_lattice(700, "sphere", radius=0.4, chi=1.0, seed=3)
    want = oracle_step(oracle, sc.pos, sc.h, sc.volume, sc.chi, sc.H0)
    s = make(mf, sc)
    s.tolerance = 1e-7
    s.max_iteration = 400
    s.solve(400)
    # the reference's absolute epsilons stall its NLCG near 1e-6 relative
    assert rel(s.total_B_over_mu0, want["b"]) < 2e-5


def test_naive_quirks(mf, oracle):
    # naive=true: external sources use h instead of ext_mag_h and the external
    # force term carries mu0 twice (magnetic_force.cu:1118, :589-600)
    import scenes
    sc = scenes.jittered_lattice(300, "sphere", radius=0.3, chi=1.0, seed=5)
    ext_p = np.float32([[0.0, 0.0, -0.6], [0.1, 0.0, 0.7]])
    ext_m = np.float32([[0.0, 0.0, 0.02], [0.0, 0.01, 0.0]])
    for naive in (False, True):
        want = oracle_step(oracle, sc.pos, sc.h, sc.volume, sc.chi, sc.H0, ext_p, ext_m, ext_h=0.2, naive=naive)
        s = make(mf, sc, ext_pos=ext_p, ext_m=ext_m, ext_h=0.2)
        s.naive = naive
        s.set_option("solver", mf.SOLVER_CG)
        s.solve(200)
        s.evaluate_fitted_near_foece()
        assert rel(s.Hext, want["hext"]) < 1e-6
        assert rel(s.M, want["M"]) < 1e-5
        assert rel(s.magnetic_bodyforce, want["F"]) < 1e-5


def test_resize_keeps_warm_start(mf):
    import scenes
    sc = scenes.jittered_lattice(1000, "sphere", radius=0.5, chi=2.0, seed=8)
    s = make(mf, sc)
    s.set_option("solver", mf.SOLVER_CG)
    s.solve(100)
    b = s.total_B_over_mu0
    s.setTargetpos(sc.pos[:600])
    assert s.np == 600
    assert np.array_equal(s.total_B_over_mu0, b[:600])
    s.setTargetpos(sc.pos)
    b2 = s.total_B_over_mu0
    assert np.array_equal(b2[:600], b[:600]) and np.all(b2[600:] == 0)


def test_advance_matches_oracle(mf, oracle):
    import scenes
    sc = scenes.jittered_lattice(400, "sphere", radius=0.5, chi=2.0, seed=9)
    s = make(mf, sc)
    s.set_option("solver", mf.SOLVER_CG)
    dt = 1e-4
    pos = sc.pos.astype(np.float64)
    vel = np.zeros_like(pos)
    for _ in range(3):
        s.advance(dt, 200)
        w = oracle_step(oracle, pos, sc.h, sc.volume, sc.chi, sc.H0)
        vel += dt * w["F"] / sc.volume
        pos += dt * vel
    assert rel(s.get("velocity"), vel) < 1e-4
    # displacements here are below the FP32 spacing of the coordinates: the
    # positions must agree to a couple of ulps
    assert np.max(np.abs(s.xyz - pos)) < 2e-7


def test_invalid_inputs(mf):
    g = main_cu_scene()
    with pytest.raises(mf.MFError) as e:
        mf.Solver(8, -1.0, 1.0, 1.0, 1.0, [0, 1, 0], None, None, g)
    assert e.value.status == 1
    s = mf.Solver(8, 1.0, 1.0, 1.0, 1.0, [0, 1, 0], None, None, g)
    bad = g.copy()
    bad[3, 1] = np.nan
    with pytest.raises(mf.MFError):
        s.setTargetpos(bad)
    with pytest.raises(mf.MFError):
        s.set_option("solver", 7)


def test_export_formats(mf, tmp_path):
    g = main_cu_scene()
    s = mf.Solver(8, 1.0, 1.0, 1.0, 1.0, [0, 1, 0], np.float32([[0, -100, 0]]), np.float32([[0, 1, 0]]), g)
    s.solve(100)
    s.evaluate_fitted_near_foece()
    p1, p2 = str(tmp_path / "temp.txt"), str(tmp_path / "force.txt")
    s.export_data(p1)
    s.export_force(p2)
    d = np.loadtxt(p1)
    f = np.loadtxt(p2)
    assert d.shape == (8, 10) and f.shape == (8, 10)
    assert np.array_equal(d[:, 0], np.arange(8))
    assert np.allclose(d[:, 1:4], g) and np.allclose(d[:, 4:7], s.total_B_over_mu0, rtol=1e-5)
    assert np.allclose(f[:, 4:7], s.magnetic_bodyforce, rtol=1e-5, atol=1e-30)
    assert np.allclose(d[:, 7:10], s.Hext, rtol=1e-5)


def test_counters(mf):
    import scenes
    sc = scenes.jittered_lattice(1024, "sphere", radius=0.5, chi=2.0, seed=2)
    s = make(mf, sc)
    s.set_option("solver", mf.SOLVER_CG)
    s.reset_counters()
    it, _ = s.solve(100)
    s.evaluate_fitted_near_foece()
    c = s.counters()
    assert c["field_products"] == it + 1
    assert c["field_pairs"] == (it + 1) * 1024 * 1024
    assert c["force_pairs"] == 1024 * 1024


def test_autotuned_shapes_match_default(mf):
    # Every block shape computes the same sums (only the FP32 order of the
    # per-tile partial sums differs): tuned and fixed-shape handles agree, and
    # both meet the oracle bar.
    import scenes
    sc = scenes.jittered_lattice(20000, "sphere", radius=0.5, chi=2.0, seed=12)
    out = {}
    for mode in (0, 1):
        s = make(mf, sc)
        s.set_option("autotune", mode)
        s.set_option("solver", mf.SOLVER_CG)
        s.solve(200)
        s.evaluate_fitted_near_foece()
        out[mode] = (s.total_B_over_mu0, s.magnetic_bodyforce)
        assert s.get_option("autotune") == mode
    assert rel(out[1][0], out[0][0]) < 1e-6
    assert rel(out[1][1], out[0][1]) < 1e-6
    rep = mf.autotune_report()
    assert any("field_packed" in ln for ln in rep) and any("force_packed" in ln for ln in rep)


@pytest.mark.parametrize("n", [14337, 32769])
def test_force_once_per_pair_matches_oracle(mf, oracle, n):
    # The packed field and force of one scene evaluated once per unordered
    # pair (T even in d, f_ji = -f_ij; MF_OPT_PAIR_SYMMETRIC 2): the kernel
    # statistics show one evaluation per unordered pair.  n is one past a
    # multiple of the kernel's block (1,024 particles), so the last block
    # holds a single particle.
    import scenes
    sc = scenes.jittered_lattice(n, "sphere", radius=0.5, chi=2.0, seed=n)
    s = make(mf, sc)
    s.set_option("pair_symmetric", 2)
    assert s.get_option("pair_symmetric") == 2
    s.set_option("solver", mf.SOLVER_CG)
    s.set_option("kernel_timing", 1)
    it, relres = s.solve(200)
    assert relres < 1e-6
    fs = s.kernel_stats("field")
    assert fs["launches"] >= 1 and fs["evals"] == fs["launches"] * float(n) * (n - 1) / 2
    s.reset_counters()
    s.evaluate_fitted_near_foece()
    st = s.kernel_stats("force")
    assert st["launches"] == 1 and st["pairs"] == float(n) * n
    assert st["evals"] == float(n) * (n - 1) / 2
    M = np.asarray(s.M, np.float64)
    F = oracle.force(np.asarray(sc.pos, np.float64), M, sc.h, None)
    got = np.asarray(s.magnetic_bodyforce, np.float64)
    assert rel(got, F) < 1e-5
    # internal forces only (uniform applied field): they sum to zero
    assert np.linalg.norm(got.sum(axis=0)) < 1e-5 * np.abs(got).sum()


@pytest.mark.parametrize("n", [2049, 5001])
def test_field_once_per_pair_matches_oracle(mf, oracle, n):
    # Packed field products once per unordered pair through a whole CG
    # solve (the launches after convergence skipped by the done flag), against
    # the FP64 oracle; and the same handle with every ordered pair evaluated
    # (MF_OPT_PAIR_SYMMETRIC 0) agrees to FP32 summation order.
    import scenes
    sc = scenes.jittered_lattice(n, "sphere", radius=0.5, chi=2.0, seed=n + 7)
    want = oracle_step(oracle, sc.pos, sc.h, sc.volume, sc.chi, sc.H0)
    out = {}
    for mode in (2, 0):
        s = make(mf, sc)
        s.set_option("pair_symmetric", mode)
        s.set_option("solver", mf.SOLVER_CG)
        s.set_option("kernel_timing", 1)
        it, relres = s.solve(200)
        assert relres < 1e-6
        st = s.kernel_stats("field")
        per = float(n) * (n - 1) / 2 if mode == 2 else float(n) * n
        assert st["evals"] == st["launches"] * per
        s.evaluate_fitted_near_foece()
        out[mode] = (np.asarray(s.total_B_over_mu0), np.asarray(s.M), np.asarray(s.magnetic_bodyforce))
        s.close()
    assert rel(out[2][0], want["b"]) < 1e-5
    assert rel(out[2][1], want["M"]) < 1e-5
    assert rel(out[2][2], want["F"]) < 1e-5
    assert rel(out[2][0], out[0][0]) < 1e-6
    assert rel(out[2][2], out[0][2]) < 1e-5
