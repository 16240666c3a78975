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
    assert r["frac_of_body_bound"] == pytest.approx(want / peak / (110.0 / 156.0), abs=1e-4)
    assert r["kernels"]["field"]["tflops"] == pytest.approx(49.0 * n * (n - 1) / 2 / 2.5e-3 / 1e12)
    # every ordered pair: the all-pairs counts
    r = bench.pair_roofline(stats(n, 2.81, 40, False), stats(n, 4.08, 40, False), peak, n)
    assert r["kernel"] == "allpairs_kernel<force>"
    assert r["achieved"] == pytest.approx(53.0 * n * n / 4.08e-3 / 1e12, abs=1e-3)
    assert r["kernels"]["field"]["body_bound"] == pytest.approx(64.0 / 76.0, abs=1e-4)


def test_traffic_only_at_the_profiled_size(bench):
    r = bench.pair_roofline(stats(32768, 1.0, 1, True), stats(32768, 1.0, 1, True), 73.0, 32768)
    assert r["traffic"] is None
