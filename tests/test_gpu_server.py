"""GPU tests of the served stream (mf_server_*): continuous batching admits
requests between timesteps; each request's final state is the same whether it
ran alone or in the mix (relative L2 within 1e-5, the FP32 bar), and the HBM
budget is enforced."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def scenes_for(sizes, seed):
    import scenes
    out = []
    for k, n in enumerate(sizes):
        rng = np.random.default_rng(seed + k)
        H = rng.normal(size=3)
        H /= np.linalg.norm(H)
        out.append(scenes.jittered_lattice(n, "sphere", radius=float(rng.uniform(0.2, 0.5)),
                                           chi=float(rng.uniform(0.5, 3.0)), seed=seed + k, H0=tuple(H)))
    return out


def run_alone(mf, sc, steps):
    srv = mf.Server(steps_per_request=steps, dt=1e-3, rel_tol=1e-7, iters_per_step=8)
    rid = srv.submit(sc)
    while srv.poll(rid)[0] != 2:
        srv.step()
    out = {q: srv.result(rid, q) for q in ("positions", "velocity", "magnetic_bodyforce", "total_B_over_mu0")}
    srv.close()
    return out


def test_alone_equals_in_the_mix(mf):
    scs = scenes_for((700, 1500, 333, 2000), seed=41)
    steps = 4
    srv = mf.Server(steps_per_request=steps, dt=1e-3, rel_tol=1e-7, iters_per_step=8)
    ids = []
    # staggered arrivals: requests join while others are running
    for k, sc in enumerate(scs):
        ids.append(srv.submit(sc))
        srv.step()
    while any(srv.poll(i)[0] != 2 for i in ids):
        srv.step()
    st = srv.stats()
    assert st["completed"] == len(scs) and st["rebatches"] >= 2
    for i in ids:
        t = srv.step_times(i)
        assert len(t) == steps and np.all(t > 0)
    for k in (0, 2, 3):
        alone = run_alone(mf, scs[k], steps)
        for q, v in alone.items():
            got = srv.result(ids[k], q)
            if q == "positions":
                assert np.max(np.abs(got - v)) < 1e-6
            else:
                assert rel(got, v) < 1e-5, (k, q, rel(got, v))
        assert srv.poll(ids[k])[1] == steps
    srv.close()


def test_budget_enforced(mf):
    import scenes
    sc = scenes.jittered_lattice(4000, "sphere", radius=0.4, chi=1.0, seed=5)
    srv = mf.Server(hbm_budget_bytes=2e6, steps_per_request=2)
    with pytest.raises(mf.MFError) as e:
        srv.submit(sc)
    assert e.value.status == 6  # MF_ERR_BUDGET
    srv.close()
    # a budget for one request at a time: the second waits in the queue
    srv = mf.Server(hbm_budget_bytes=4000 * 320 + 4.2 * 1024 * 1024, steps_per_request=2)
    a, b = srv.submit(sc), srv.submit(sc)
    srv.step()
    assert srv.poll(a)[0] == 1 and srv.poll(b)[0] == 0
    while srv.poll(b)[0] != 2:
        srv.step()
    assert srv.poll(a)[0] == 2
    srv.close()


def test_fmm_request_in_the_mix(mf, oracle):
    # A request above 65,536 particles runs as its own solver handle (field
    # products through the FMM at P = 8, the force as the handle's automatic
    # choice picks it) on a host thread and a stream of its own beside the
    # batch; its result equals the same solver run alone with the same
    # settings, is within 1e-5 of FP64 oracle sums, and the small requests
    # are unaffected.
    import scenes
    big = scenes.jittered_lattice(70000, "cylinder", radius=0.3, height=1.0, chi=1.5, seed=77)
    small = scenes_for((900, 1700), seed=51)
    steps = 3
    srv = mf.Server(steps_per_request=steps, dt=1e-3, rel_tol=1e-7, iters_per_step=8)
    ids = [srv.submit(small[0]), srv.submit(big)]
    srv.step()
    ids.append(srv.submit(small[1]))
    while any(srv.poll(i)[0] != 2 for i in ids):
        srv.step()
    st = srv.stats()
    assert st["completed"] == 3 and st["force_pairs"] > 0
    # the FMM request took its timesteps on its own thread, each timed
    t = srv.step_times(ids[1])
    assert len(t) == steps and np.all(t > 0)
    # the big request against a standalone FMM solver with the server's settings
    s = mf.Solver(big.n, big.h, big.h, big.volume, big.chi, big.H0, None, None, big.pos)
    s.set_option("solver", mf.SOLVER_CG)
    s.set_option("rel_tol", 1e-7)
    s.solve(500)
    for _ in range(steps):
        s.advance(1e-3, 8)
    assert s.fmm_stats()["active"] == 1
    assert np.max(np.abs(srv.result(ids[1], "positions") - s.xyz)) < 1e-6
    assert rel(srv.result(ids[1], "magnetic_bodyforce"), s.magnetic_bodyforce) < 1e-5
    assert rel(srv.result(ids[1], "total_B_over_mu0"), s.total_B_over_mu0) < 1e-5
    # The same handle solved and its force evaluated at the final positions
    # (a timestep ends by moving the particles), against FP64 oracle sums
    # over all N at 512 particles: the fixed-point residual of b and the
    # force at its M.
    s.solve(500)
    s.evaluate_fitted_near_foece()
    idx = np.sort(np.random.default_rng(3).choice(big.n, 512, replace=False))
    pos = np.asarray(s.xyz, np.float64)
    b = np.asarray(s.total_B_over_mu0, np.float64)
    M = np.asarray(s.M, np.float64)
    G = oracle.field(pos[idx], pos, M, big.h)
    H0 = np.tile(np.asarray(big.H0, np.float64), (len(idx), 1))
    res = np.linalg.norm(b[idx] - H0 - G) / np.linalg.norm(H0)
    T = oracle.tensor_sum(pos[idx], pos, M, big.h).reshape(-1, 3, 3)
    F = np.einsum("icr,ic->ir", T, M[idx])
    ef = rel(s.magnetic_bodyforce[idx], F)
    assert res < 1e-5 and ef < 1e-5, (res, ef)
    for k, sc in ((0, small[0]), (2, small[1])):
        alone = run_alone(mf, sc, steps)
        assert rel(srv.result(ids[k], "magnetic_bodyforce"), alone["magnetic_bodyforce"]) < 1e-5
    srv.close()


def test_submit_rejects_bad_scenes(mf):
    # Bad parameters are refused at submission, before they can fail a batch
    # rebuild or an FMM request's thread; the server keeps serving.
    import dataclasses
    import scenes
    sc = scenes.jittered_lattice(1000, "sphere", radius=0.3, chi=1.0, seed=7)
    srv = mf.Server(steps_per_request=2)
    for bad in (dict(h=0.0), dict(h=float("nan")), dict(volume=-1.0), dict(chi=-1.0), dict(chi=float("inf")),
                dict(H0=(0.0, float("nan"), 1.0))):
        with pytest.raises(mf.MFError) as e:
            srv.submit(dataclasses.replace(sc, **bad))
        assert e.value.status == 1  # MF_ERR_INVALID_ARG
    rid = srv.submit(sc)
    while srv.poll(rid)[0] != 2:
        srv.step()
    assert srv.stats()["completed"] == 1
    srv.close()
