"""CPU checks of bench.py's roofline arithmetic (no GPU): the algorithmic FLOP
of each product kind, ordered pairs for the all-pairs kernels and unordered
pairs for the products evaluated once per pair, and the fractions of the
measured peak and of the body's FMA-pipe ceiling."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench as b
    return b


def stats(n, ms, launches, once_per_pair):
    pairs = float(n) * n * launches
    evals = float(n) * (n - 1) / 2 * launches if once_per_pair else pairs
    return {"launches": launches, "total_ms": ms * launches, "pairs": pairs, "evals": evals}


def test_ordered_and_unordered_counts(bench):
    n, peak = 65536, 73.0
    kf = stats(n, 2.5, 40, True)
    kg = stats(n, 2.9, 40, True)
    r = bench.pair_roofline(kf, kg, peak, n)
    assert r["kernel"] == "k_sym<force>"  # the longer product
    f = r["kernels"]["force"]
    want = 55.0 * n * (n - 1) / 2 / 2.9e-3 / 1e12
    assert f["tflops"] == pytest.approx(want)
    assert r["frac"] == pytest.approx(want / peak, abs=1e-4)
    assert r["frac_of_body_bound"] == pytest.approx(want / peak / (110.0 / 144.0), abs=1e-4)
    assert r["kernels"]["field"]["tflops"] == pytest.approx(49.0 * n * (n - 1) / 2 / 2.5e-3 / 1e12)
    # every ordered pair: the all-pairs counts
    r = bench.pair_roofline(stats(n, 2.81, 40, False), stats(n, 4.08, 40, False), peak, n)
    assert r["kernel"] == "allpairs_kernel<force>"
    assert r["achieved"] == pytest.approx(53.0 * n * n / 4.08e-3 / 1e12, abs=1e-3)
    assert r["kernels"]["field"]["body_bound"] == pytest.approx(64.0 / 76.0, abs=1e-4)


def test_field_and_force_in_one_launch(bench):
    # Steps whose solve keeps its warm start: one fused launch per step, the
    # shared terms counted once (86 FLOP per unordered pair).
    n, peak = 65536, 80.5
    kff = stats(n, 4.5, 10, True)
    kff["pairs"] *= 2  # both products' pairs
    none = {"launches": 0, "total_ms": 0.0, "pairs": 0.0, "evals": 0.0}
    r = bench.pair_roofline(none, none, peak, n, kff=kff)
    assert r["kernel"] == "k_sym_ff<field+force>"
    want = 86.0 * n * (n - 1) / 2 / 4.5e-3 / 1e12
    assert r["achieved"] == pytest.approx(want, abs=1e-3)
    assert r["kernels"]["field_force"]["body_bound"] == pytest.approx(172.0 / 216.0, abs=1e-4)
    assert set(r["kernels"]) == {"field_force"}
    # the same launch at the two products' own counts (49 + 55)
    assert r["kernels"]["field_force"]["tflops_at_product_counts"] == pytest.approx(want * 104.0 / 86.0)
    # the profiled DRAM bytes of this launch at this size
    assert r["traffic"] == 43090688


def test_traffic_only_at_the_profiled_size(bench):
    r = bench.pair_roofline(stats(32768, 1.0, 1, True), stats(32768, 1.0, 1, True), 73.0, 32768)
    assert r["traffic"] is None


def test_comparison_summaries(bench):
    # The batched-vs-plain and served-vs-plain records carried on the default
    # line: the ratios are the batched / served pairs/s over the plain ones.
    batch = {"value": 1.0e12, "ms_per_step": 76.0, "p50_step_ms": 76.1, "p99_step_ms": 76.4, "steps": 5,
             "gpu_launches": 70, "max_iters_last_step": 0.0, "batched_over_plain": 1.0e12 / 4.4e11,
             "plain": {"value": 4.4e11, "ms_per_step": 174.0, "passes": 1}, "config": {"workload": "batch256"},
             "clocks": {"sm_mhz": 2070.0}}
    b = bench.summarize_batch(batch)
    assert b["ratio"] == pytest.approx(1.0e12 / 4.4e11)
    assert b["batched"]["ms_per_step"] == 76.0 and b["plain"]["ms_per_step"] == 174.0
    keys = ("value", "unit", "p50_step_ms", "p99_step_ms", "p50_request_ms", "p99_request_ms")
    plain = dict(zip(keys, (1.0e12, "pairs/s", 1.2, 120.0, 2300.0, 3300.0)), capacity_req_per_s=3.6)
    served = dict(zip(keys, (1.1e12, "pairs/s", 12.0, 220.0, 950.0, 3900.0)))
    served.update({"requests": 24, "rate_per_s": 3.9, "rate_basis": "80 %", "capacity_req_per_s": 4.9,
                   "n_range": [1282, 224677], "p50_tick_ms": 3.0, "p99_tick_ms": 180.0, "step_ms_by_path": {},
                   "clocks": {}, "note": "", "plain": plain})
    v = bench.summarize_served(served)
    assert v["ratio"] == pytest.approx(1.1) and v["capacity_ratio"] == pytest.approx(4.9 / 3.6)
    assert v["served"]["p99_step_ms"] == 220.0 and v["plain"]["p99_step_ms"] == 120.0
    served["plain"] = None
    assert bench.summarize_served(served)["ratio"] is None


def test_both_arms_share_the_config(bench):
    class A:
        dt, rel_tol = 1e-4, 1e-6
    c = bench.config_allpairs(65536, 0.04, A())
    assert c["N"] == 65536 and "allpairs_fp32_65536" in c["workload"] and "rel tol 1e-06" in c["workload"]
