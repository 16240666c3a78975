"""GPU tests of the FMM path (uniform octree, Cartesian expansions) against
the FP64 direct oracle and against the handle's own all-pairs path.

The FMM's only approximation is the expansion truncation: every far box pair
is beyond the kernel's near radius, so the reference's SPH / fitted-curve
near field is evaluated exactly.  Tolerances (relative L2 over all sampled
particles and components):
  field operator G(m), P = 8, aperture 0.5           1e-5  (measured 2e-6 .. 3e-6)
  Kelvin force / force tensor, P = 10, aperture 0.44  1e-5  (measured 4e-6 .. 6e-6; at 0.5 it
                                                           is 6e-5 .. 1.3e-4: the Hessian of the
                                                           local expansion, relative to the small
                                                           net force of a magnetised body)
  solved B/mu0 and M, P = 8                          1e-5
  field operator, P = 6 (not the default)            1e-4  (measured 3e-5: P = 6 does not meet
                                                           1e-5 at aperture 0.5)
  theta -> 0 (every box near): FMM = all-pairs up to summation order, 2e-6
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def solver(mf, sc, **opts):
    s = mf.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos, precision="fp32")
    for k, v in opts.items():
        s.set_option(k, v)
    return s


def moments(sc, seed=1):
    rng = np.random.default_rng(seed)
    return (np.array([0.2, -0.1, 1.0]) + 0.3 * rng.standard_normal((sc.n, 3))) * sc.volume


@pytest.fixture(scope="module")
def sphere40k():
    import scenes
    return scenes.jittered_lattice(40000, "sphere", radius=0.5, chi=1.5, seed=3)


@pytest.fixture(scope="module")
def cylinder100k():
    import scenes
    return scenes.jittered_lattice(100000, "cylinder", radius=0.3, height=1.0, chi=1.5, seed=3)


@pytest.mark.parametrize("order,leaf,tol", [(8, 8, 1e-5), (6, 8, 1e-4), (8, 64, 1e-5), (5, 16, 3e-4)])
def test_field_operator_vs_oracle(mf, oracle, sphere40k, order, leaf, tol):
    sc = sphere40k
    m = moments(sc)
    rng = np.random.default_rng(2)
    idx = rng.choice(sc.n, 1500, replace=False)
    want = oracle.field(sc.pos[idx].astype(np.float64), sc.pos.astype(np.float64), m, sc.h)
    s = solver(mf, sc, fmm=mf.FMM_ON, fmm_order=order, fmm_leaf=leaf)
    got = s.apply_field(m)
    st = s.fmm_stats()
    assert st["active"] == 1 and st["degree"] == order - 1
    assert rel(got[idx], want) < tol


def test_field_operator_cylinder(mf, oracle, cylinder100k):
    sc = cylinder100k
    m = moments(sc, seed=4)
    idx = np.random.default_rng(5).choice(sc.n, 1000, replace=False)
    want = oracle.field(sc.pos[idx].astype(np.float64), sc.pos.astype(np.float64), m, sc.h)
    s = solver(mf, sc, fmm=mf.FMM_ON, fmm_order=8, fmm_leaf=32)
    assert rel(s.apply_field(m)[idx], want) < 1e-5
    # the same handle on the all-pairs path
    s.set_option("fmm", mf.FMM_OFF)
    assert rel(s.apply_field(m)[idx], want) < 1e-6


def test_all_near_equals_allpairs(mf, sphere40k):
    # With a tiny aperture no box pair is accepted: the product is the near
    # field alone (packed pairs + correction) over every leaf box.
    sc = sphere40k
    m = moments(sc, seed=6)
    s = solver(mf, sc, fmm=mf.FMM_ON, fmm_theta=0.02, fmm_leaf=64)
    got = s.apply_field(m)
    st = s.fmm_stats()
    assert st["m2l_per_product"] == 0
    assert st["p2p_pairs"] == float(sc.n) * sc.n
    s.set_option("fmm", mf.FMM_OFF)
    assert rel(got, s.apply_field(m)) < 2e-6


def test_solve_and_force_vs_allpairs(mf, sphere40k):
    sc = sphere40k
    out = {}
    for mode in (mf.FMM_ON, mf.FMM_OFF):
        s = solver(mf, sc, fmm=mode, fmm_order=8, fmm_leaf=8, solver=mf.SOLVER_CG)
        it, rr = s.solve(300)
        assert rr < 1e-6
        s.evaluate_fitted_near_foece()
        out[mode] = (s.total_B_over_mu0, s.M, s.magnetic_bodyforce)
        if mode == mf.FMM_ON:
            st = s.fmm_stats()
            assert st["field_products"] >= it and st["force_products"] == 1
    b1, m1, f1 = out[mf.FMM_ON]
    b2, m2, f2 = out[mf.FMM_OFF]
    assert rel(b1, b2) < 1e-5
    assert rel(m1, m2) < 1e-5
    assert rel(f1, f2) < 1e-5


def test_nlcg_with_fmm(mf, sphere40k):
    sc = sphere40k
    s = solver(mf, sc, fmm=mf.FMM_ON, fmm_order=6, fmm_leaf=16)
    s.tolerance = 1e-4
    s.solve(40)
    h = s.error_history()
    assert len(h) >= 2 and h[-1] < h[0]


def test_advance_rebuilds_tree(mf, cylinder100k):
    # Positions move each step; the octree is rebuilt from the new positions.
    sc = cylinder100k
    res = {}
    for mode in (mf.FMM_ON, mf.FMM_OFF):
        s = solver(mf, sc, fmm=mode, fmm_order=8, fmm_leaf=32, solver=mf.SOLVER_CG)
        for _ in range(2):
            s.advance(1e-3, 100)
        res[mode] = (s.xyz, s.magnetic_bodyforce)
    assert np.max(np.abs(res[mf.FMM_ON][0] - res[mf.FMM_OFF][0])) < 1e-6
    assert rel(res[mf.FMM_ON][1], res[mf.FMM_OFF][1]) < 1e-5


def test_auto_mode_threshold(mf):
    # Field products through the FMM above 65,536 particles, the Kelvin force
    # above 90,000 (below, its wider near field covers most of the scene).
    import scenes
    small = scenes.uniform_cube(65536, seed=9, volume=1e-6, chi=1.0)
    big = scenes.uniform_cube(65537, seed=9, volume=1e-6, chi=1.0)
    huge = scenes.uniform_cube(262145, seed=9, volume=1e-6, chi=1.0)
    st = solver(mf, small, autotune=0).fmm_stats()
    assert st["active"] == 0 and st["force_active"] == 0
    st = solver(mf, big, autotune=0).fmm_stats()
    assert st["active"] == 1 and st["force_active"] == 0
    st = solver(mf, huge, autotune=0).fmm_stats()
    assert st["active"] == 1 and st["force_active"] == 1
    s = solver(mf, big, fmm=mf.FMM_OFF)
    assert s.fmm_stats()["active"] == 0


def test_bad_fmm_options(mf, sphere40k):
    s = solver(mf, sphere40k)
    for key, v in (("fmm", 3), ("fmm_order", 3), ("fmm_order", 10), ("fmm_theta", 0.0), ("fmm_theta", 1.5),
                   ("fmm_leaf", 0), ("fmm_force_theta", 0.0), ("fmm_force_theta", 1.01), ("fmm_force_order", 3),
                   ("fmm_force_order", 11), ("fmm_force_order", 8.5)):
        with pytest.raises(mf.MFError):
            s.set_option(key, v)


def _raw_scene(pos, h, chi=1.0):
    import scenes
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    return scenes.Scene(pos=pos, h=h, volume=h ** 3 / 8, chi=chi, H0=(0.0, 0.0, 1.0), spacing=h / 2, meta={})


@pytest.mark.parametrize("kind", ["plane", "line", "two_clusters", "tiny"])
def test_degenerate_geometry(mf, kind):
    # Flat and thin bounding boxes, far-apart clusters (mostly empty grid) and
    # a scene smaller than one leaf: the FMM still equals all-pairs to its
    # truncation error.
    rng = np.random.default_rng(17)
    if kind == "plane":
        g = np.stack(np.meshgrid(np.arange(160), np.arange(160), indexing="ij"), -1).reshape(-1, 2) * 0.01
        pos = np.c_[g + rng.uniform(-0.002, 0.002, g.shape), np.zeros(len(g))]
        h = 0.02
    elif kind == "line":
        x = np.arange(6000) * 0.01
        pos = np.c_[x, rng.uniform(-0.001, 0.001, (6000, 2))]
        h = 0.02
    elif kind == "two_clusters":
        a = rng.uniform(-0.1, 0.1, (15000, 3))
        pos = np.r_[a, a + np.array([3.0, 0.5, -1.0])]
        h = 0.016
    else:
        pos = rng.uniform(0, 0.2, (50, 3))
        h = 0.05
    sc = _raw_scene(pos, h)
    m = moments(sc, seed=3)
    s = solver(mf, sc, fmm=mf.FMM_ON, fmm_order=8, fmm_leaf=32)
    got = s.apply_field(m)
    assert np.all(np.isfinite(got))
    st = s.fmm_stats()
    assert st["active"] == 1 and st["occupied_leaves"] >= 1
    s.set_option("fmm", mf.FMM_OFF)
    assert rel(got, s.apply_field(m)) < 1e-5


def test_fmm_matrix_separate_targets(mf, oracle, sphere40k):
    # The kernel_matrix form: sources and a separate target set (inside,
    # around and far from the sources, some on source positions).
    sc = sphere40k
    rng = np.random.default_rng(8)
    tg = np.r_[rng.uniform(-0.6, 0.6, (3000, 3)), sc.pos[:500], rng.uniform(2.0, 2.5, (200, 3))].astype(np.float32)
    m = moments(sc, seed=9)
    A = mf.FmmMatrix(sc.pos, sc.h, targets=tg, order=8, theta=0.5, leaf_min=16)
    got = A.field(m)
    want = oracle.field(tg.astype(np.float64), sc.pos.astype(np.float64), m, sc.h)
    assert rel(got, want) < 1e-5
    st = A.stats()
    assert st["active"] == 1 and st["m2l_per_product"] > 0
    # a second product on the same matrix with new charges
    m2 = moments(sc, seed=10)
    want2 = oracle.field(tg.astype(np.float64), sc.pos.astype(np.float64), m2, sc.h)
    assert rel(A.field(m2), want2) < 1e-5
    A.close()


def test_fmm_matrix_same_targets(mf, sphere40k):
    sc = sphere40k
    m = moments(sc, seed=11)
    A = mf.FmmMatrix(sc.pos, sc.h, order=8, leaf_min=16)
    s = solver(mf, sc, fmm=mf.FMM_ON, fmm_order=8, fmm_leaf=16)
    assert rel(A.field(m), s.apply_field(m)) < 1e-6
    A.close()


def test_fmm_matrix_hessian(mf, oracle, sphere40k):
    # The kernel_matrix<DipoleHessianSpherical> form: 3x3 force tensors at a
    # separate target set, glm column-major like mf_direct_force_tensor.
    sc = sphere40k
    rng = np.random.default_rng(12)
    tg = np.r_[rng.uniform(-0.55, 0.55, (1500, 3)), sc.pos[:300]].astype(np.float32)
    m = moments(sc, seed=13)
    A = mf.FmmMatrix(sc.pos, sc.h, targets=tg, order=8, theta=0.5, leaf_min=16)
    got = A.hessian(m)
    want = oracle.tensor_sum(tg.astype(np.float64), sc.pos.astype(np.float64), m, sc.h).reshape(-1, 9)
    assert got.shape == (len(tg), 9)
    assert rel(got, want) < 1e-5
    st = A.stats()
    assert st["theta"] == 0.5 and abs(st["force_theta"] - 0.44) < 1e-12
    assert st["force_p2p_pairs"] >= st["p2p_pairs"]  # equal where the leaf boxes make them so
    # symmetric 3x3 per target
    g3 = got.reshape(-1, 3, 3)
    assert np.allclose(g3, np.transpose(g3, (0, 2, 1)), rtol=0, atol=1e-6 * np.abs(g3).max())
    A.close()


def test_many_external_dipoles_through_fmm(mf):
    # More than 65,536 external dipoles: H_ext and its gradient tensor come
    # from an octree over the external sources (the particles as separate
    # targets, smoothing length ext_mag_h), and equal the all-pairs
    # evaluation of the same handle to the FMM's truncation error.
    import scenes
    sc = scenes.jittered_lattice(8000, "sphere", radius=0.3, chi=1.5, seed=21)
    rng = np.random.default_rng(22)
    ne = 70000
    src = rng.uniform(-0.7, 0.7, (ne, 3)).astype(np.float32)
    mom = ((np.array([0.0, 0.2, 1.0]) + 0.3 * rng.standard_normal((ne, 3))) * sc.volume).astype(np.float32)
    hext = 2.0 * sc.h
    out = {}
    for mode in (mf.FMM_ON, mf.FMM_OFF):
        s = mf.Solver(sc.n, sc.h, hext, sc.volume, sc.chi, sc.H0, src, mom, sc.pos, precision="fp32")
        s.set_option("solver", mf.SOLVER_CG)
        s.set_option("fmm", mode)
        s.set_option("fmm_order", 8)
        s.solve(300)
        out[mode] = (s.Hext, np.stack([s.dHextdx, s.dHextdy, s.dHextdz]), s.total_B_over_mu0)
    h1, g1, b1 = out[mf.FMM_ON]
    h2, g2, b2 = out[mf.FMM_OFF]
    e = rel(h1 - np.asarray(sc.H0, np.float32), h2 - np.asarray(sc.H0, np.float32))
    # the two paths differ (the all-pairs one is deterministic, so equality
    # would mean the FMM did not run) by no more than the truncation error
    assert 0.0 < e < 1e-5
    assert rel(g1, g2) < 1e-5
    assert rel(b1, b2) < 1e-5


@pytest.mark.parametrize("leaf", [8, 200])
def test_force_near_field_once_per_box_pair(mf, sphere40k, leaf):
    # The FMM's near field of the force once per unordered box pair
    # (MF_OPT_PAIR_SYMMETRIC 2; the default from 1,048,576 particles) against
    # every ordered pair (0):
    # the magnetization and the far field are the same, the near sums differ
    # in FP32 order only.  leaf 200 makes boxes of more than 128 particles
    # (more than one target round per warp).
    sc = sphere40k
    out = {}
    for mode in (2, 0):
        s = solver(mf, sc, fmm=mf.FMM_ON, fmm_order=8, fmm_leaf=leaf, solver=mf.SOLVER_CG)
        s.set_option("pair_symmetric", mode)
        it, rr = s.solve(300)
        assert rr < 1e-6
        s.set_option("kernel_timing", 1)
        s.reset_counters()
        s.evaluate_fitted_near_foece()
        out[mode] = (np.asarray(s.magnetic_bodyforce, np.float64), s.kernel_stats("fmm_near_force"),
                     s.fmm_stats()["max_leaf"])
        s.close()
    sym, full = out[2][1], out[0][1]
    assert full["evals"] == full["pairs"]
    assert sym["pairs"] == full["pairs"] and 0.45 * sym["pairs"] < sym["evals"] < 0.6 * sym["pairs"]
    if leaf == 200:
        assert out[2][2] > 128
    assert rel(out[2][0], out[0][0]) < 2e-6


@pytest.fixture(scope="module")
def cylinder262k():
    import scenes
    return scenes.config_fmm_1m(262144)


def test_reduced_cylinder_config_vs_oracle(mf, oracle, cylinder262k):
    # The 1,048,576-particle cylinder's shape at a quarter of its particles
    # (r = 0.3, height 1, h = 2 spacings, chi = 1.5), both products through
    # the FMM at the defaults.  Against FP64 oracle sums over all N at 1,024
    # seeded particles, with the handle's own magnetization:
    #   fixed-point residual |b - Hext - G(M)| / |Hext|  (the solve's accuracy)
    #   field operator G(M) and the Kelvin force at M.
    sc = cylinder262k
    s = solver(mf, sc, fmm=mf.FMM_ON, solver=mf.SOLVER_CG, rel_tol=1e-7)
    it, rr = s.solve(300)
    assert rr < 1e-7
    s.evaluate_fitted_near_foece()
    st = s.fmm_stats()
    assert st["active"] == 1 and st["force_active"] == 1 and st["degree"] == 7
    idx = np.sort(np.random.default_rng(31).choice(sc.n, 1024, replace=False))
    p64 = sc.pos.astype(np.float64)
    M = np.asarray(s.M, np.float64)
    b = np.asarray(s.total_B_over_mu0, np.float64)
    hext = np.asarray(s.Hext, np.float64)
    G = oracle.field(p64[idx], p64, M, sc.h)
    res = np.linalg.norm(b[idx] - hext[idx] - G) / np.linalg.norm(hext[idx])
    eg = rel(s.apply_field(M)[idx], G)
    T = oracle.tensor_sum(p64[idx], p64, M, sc.h).reshape(-1, 3, 3)
    F = np.einsum("icr,ic->ir", T, M[idx])
    ef = rel(s.magnetic_bodyforce[idx], F)
    assert res < 1e-5 and eg < 1e-5 and ef < 1e-5, (res, eg, ef)
    s.close()


def test_force_aperture_option(mf, sphere40k):
    # MF_OPT_FMM_FORCE_THETA sets the force's lists; at the field's aperture
    # the force shares the field's lists (and is less accurate).
    sc = sphere40k
    s = solver(mf, sc, fmm=mf.FMM_ON, fmm_leaf=16)
    assert s.get_option("fmm_force_theta") == 0.44 and s.get_option("fmm_order") == 8
    assert s.get_option("fmm_force_order") == 10
    s.set_option("fmm_force_theta", 0.3)
    a = s.fmm_stats()
    s.set_option("fmm_force_theta", 0.5)
    b = s.fmm_stats()
    assert a["force_p2p_pairs"] > b["force_p2p_pairs"] == b["p2p_pairs"]
    s.set_option("fmm_theta", 0.25)  # the force takes the smaller aperture
    assert s.fmm_stats()["force_theta"] == 0.25
    s.close()
