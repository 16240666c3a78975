"""Kernel-level timing of the all-pairs launches (also the small case used for
Nsight Compute captures).

    python magnetic-force_gb300/microbench.py --kernel field --n 65536 --reps 5

Runs mf_direct_field / mf_direct_force / mf_direct_force_tensor on a seeded
jittered-lattice sphere of N particles (h = 2 x spacing) with random dipoles,
times each launch with CUDA events and prints one JSON line per kernel:
device ms per call (packing included), pairs/s and algorithmic TFLOP/s.

    python magnetic-force_gb300/microbench.py --kernel fmm_field --n 262144 --reps 3

``fmm_field`` / ``fmm_force`` run FMM products (P = 8, theta = 0.5, the force at
its own aperture 0.3; --pair-symmetric 2 for the force's near field once per
unordered box pair) on a seeded
jittered-lattice cylinder (r = 0.3, height 1) of N particles: the field
operator G(m) through mf_apply_field, the force through mf_eval_force after a
CG solve; per-stage device times come from the handle's event timing.

    python magnetic-force_gb300/microbench.py --kernel fmm_step --n 1048576 --reps 1

``--density-of 1048576 --n 131072`` keeps the spacing of the 1,048,576-particle
cylinder in one of half its radius and height: the same leaf boxes (one level
higher) and near lists, an eighth of the particles (a small case for captures).

``fmm_step`` runs whole timesteps (mf_advance: octree rebuild from the moved
positions, CG solve, force) of the same cylinder through the FMM, so a
capture sees the tree and expansion passes as well as the products.

    python magnetic-force_gb300/microbench.py --kernel batch --reps 2

``batch`` runs the batched bench's 256 scenes (512..32,768 particles): cold
solve, three graph-captured warm-up timesteps, then --reps timesteps without
the graph (so a capture lists every launch) inside the profiler range.

    python magnetic-force_gb300/microbench.py --kernel engine_field --n 65536 --reps 5

``engine_field`` / ``engine_force`` run the all-pairs products of a Solver
handle (the same jittered-lattice sphere, FP32, block shapes from the
autotuner) with the handle's event timing: G(m) through mf_apply_field and
the force through mf_eval_force.  This is the launch shape the solver and
the bench use.

    python magnetic-force_gb300/microbench.py --kernel engine_step --n 65536 --reps 5 --fused 1

``engine_step`` runs warm solves and forces of a Solver handle (CG, the
positions unchanged, so every solve keeps its warm start): with --fused 1 or 2
the solve's residual and the force come from one launch (k_sym_ff), with
--fused 0 from the separate products.  It prints the device ms per step of
each kernel kind from the handle's event timing.

Every mode brackets its measured repetitions with the CUDA profiler range
(cudaProfilerStart / cudaProfilerStop), so an Nsight Compute capture given
``--profile-from-start off`` sees those launches only, not the warm-up or
tuning launches.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

FLOP = {"field": 32.0, "force": 53.0, "tensor": 53.0}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", default="field", choices=["field", "force", "tensor", "all", "fmm_field", "fmm_force", "fmm_step", "batch",
                                                      "engine_field", "engine_force", "engine_step"])
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--pair-symmetric", type=int, default=-1,
                    help="fmm_* / engine_*: MF_OPT_PAIR_SYMMETRIC of the handle (-1: its default)")
    ap.add_argument("--fused", type=int, default=-1,
                    help="engine_step: MF_OPT_FUSED_PRODUCTS of the handle (-1: its default)")
    ap.add_argument("--density-of", type=int, default=0,
                    help="fmm_*: keep the particle spacing of the cylinder of this many particles (r 0.3, "
                         "height 1) and scale its radius and height to --n particles (0: r 0.3, height 1)")
    args = ap.parse_args()

    import numpy as np
    import torch

    import mfgb
    import scenes

    if args.kernel.startswith("fmm"):
        return fmm(args, np, torch, mfgb, scenes)
    if args.kernel == "engine_step":
        return engine_step(args, np, torch, mfgb, scenes)
    if args.kernel.startswith("engine"):
        return engine(args, np, torch, mfgb, scenes)
    if args.kernel == "batch":
        return batch(args, torch, mfgb, scenes)
    sc = scenes.jittered_lattice(args.n, "sphere", radius=0.5, chi=2.0, seed=1)
    rng = np.random.default_rng(2)
    m = (rng.normal(size=(sc.n, 3)) * sc.volume).astype(np.float32)
    x = torch.from_numpy(sc.pos).cuda()
    mt = torch.from_numpy(m).cuda()
    kinds = ["field", "force", "tensor"] if args.kernel == "all" else [args.kernel]
    for kind in kinds:
        def call():
            if kind == "field":
                return mfgb.direct_field(x, x, mt, sc.h)
            if kind == "force":
                return mfgb.direct_force(x, mt, sc.h)
            return mfgb.direct_force_tensor(x, x, mt, sc.h)

        for _ in range(args.warmup):
            call()
        times = []
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        for _ in range(args.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            call()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.profiler.stop()
        best = min(times)
        pairs = float(sc.n) * sc.n
        print(json.dumps({"kernel": kind, "n": sc.n, "ms_best": best, "ms_all": times,
                          "pairs_per_s": pairs / (best * 1e-3),
                          "tflops": FLOP[kind] * pairs / (best * 1e-3) / 1e12}), flush=True)


def fmm(args, np, torch, mfgb, scenes):
    f = (args.n / args.density_of) ** (1.0 / 3.0) if args.density_of > 0 else 1.0
    sc = scenes.jittered_lattice(args.n, "cylinder", radius=0.3 * f, height=f, chi=1.5, seed=1)
    s = mfgb.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos)
    s.set_option("fmm", mfgb.FMM_ON)
    s.set_option("fmm_order", 8)
    s.set_option("solver", mfgb.SOLVER_CG)
    if args.pair_symmetric >= 0:
        s.set_option("pair_symmetric", args.pair_symmetric)
    rng = np.random.default_rng(2)
    m = ((np.array([0.0, 0.0, 1.0]) + 0.3 * rng.normal(size=(sc.n, 3))) * sc.volume).astype(np.float32)
    if args.kernel == "fmm_force":
        s.solve(200)
    if args.kernel == "fmm_step":
        return fmm_step(args, s, sc, torch)
    for _ in range(args.warmup):
        s.apply_field(m) if args.kernel == "fmm_field" else s.evaluate_fitted_near_foece()
    s.set_option("kernel_timing", 1)
    s.reset_counters()
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    for _ in range(args.reps):
        s.apply_field(m) if args.kernel == "fmm_field" else s.evaluate_fitted_near_foece()
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    kind = "field" if args.kernel == "fmm_field" else "force"
    whole = s.kernel_stats(kind)
    near = s.kernel_stats("fmm_near_" + kind)
    far = s.kernel_stats("fmm_far")
    st = s.fmm_stats()
    r = max(whole["launches"], 1)
    print(json.dumps({"kernel": args.kernel, "n": sc.n, "product_ms": whole["total_ms"] / r,
                      "near_ms": near["total_ms"] / r, "far_ms": far["total_ms"] / r,
                      "near_pairs": st["p2p_pairs"], "m2l": st["m2l_per_product"],
                      "near_tflops": FLOP[kind] * st["p2p_pairs"] / (near["total_ms"] / r * 1e-3) / 1e12,
                      "effective_pairs_per_s": float(sc.n) ** 2 / (whole["total_ms"] / r * 1e-3),
                      "fmm": st}), flush=True)


def fmm_step(args, s, sc, torch):
    s.solve(200)
    for _ in range(args.warmup):
        s.advance(1e-4, 500)
    s.set_option("kernel_timing", 1)
    s.reset_counters()
    torch.cuda.synchronize()
    times = []
    torch.cuda.profiler.start()
    for _ in range(args.reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        s.advance(1e-4, 500)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.profiler.stop()
    print(json.dumps({"kernel": args.kernel, "n": sc.n, "step_ms": times, "counters": s.counters()}), flush=True)


def batch(args, torch, mfgb, scenes):
    import time
    b = mfgb.Batch(scenes.batched_scenes(256, seed=7))
    b.solve(500, 1e-6)
    b.advance(1e-4, 3, iters_per_step=4, rel_tol=1e-6, graph=True)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    b.advance(1e-4, args.reps, iters_per_step=4, rel_tol=1e-6, graph=False)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / max(args.reps, 1)
    torch.cuda.profiler.stop()
    print(json.dumps({"kernel": "batch", "scenes": 256, "ms_per_step": ms, "counters": b.counters(),
                      "autotune": mfgb.autotune_report()}), flush=True)


def engine(args, np, torch, mfgb, scenes):
    sc = scenes.jittered_lattice(args.n, "sphere", radius=0.5, chi=2.0, seed=1)
    s = mfgb.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos)
    s.set_option("fmm", mfgb.FMM_OFF)
    if args.pair_symmetric >= 0:
        s.set_option("pair_symmetric", args.pair_symmetric)
    rng = np.random.default_rng(2)
    m = ((np.array([0.0, 0.0, 1.0]) + 0.3 * rng.normal(size=(sc.n, 3))) * sc.volume).astype(np.float32)
    field = args.kernel == "engine_field"
    if not field:
        s.solve(50)
    for _ in range(args.warmup):
        s.apply_field(m) if field else s.evaluate_fitted_near_foece()
    s.set_option("kernel_timing", 1)
    s.reset_counters()
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    for _ in range(args.reps):
        s.apply_field(m) if field else s.evaluate_fitted_near_foece()
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    kind = "field" if field else "force"
    st = s.kernel_stats(kind)
    r = max(st["launches"], 1)
    ms = st["total_ms"] / r
    pairs = float(sc.n) * sc.n
    # once per unordered pair: 49 (field) / 55 (force) FLOP per evaluation
    sym = st["evals"] < st["pairs"]
    flop = (55.0 if kind == "force" else 49.0) * st["evals"] / r if sym else FLOP[kind] * pairs
    print(json.dumps({"kernel": args.kernel, "n": sc.n, "kernel_ms": ms, "pairs_per_s": pairs / (ms * 1e-3),
                      "symmetric": sym, "tflops": flop / (ms * 1e-3) / 1e12,
                      "autotune": mfgb.autotune_report()}), flush=True)


def engine_step(args, np, torch, mfgb, scenes):
    sc = scenes.jittered_lattice(args.n, "sphere", radius=0.5, chi=2.0, seed=1)
    s = mfgb.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos)
    s.set_option("fmm", mfgb.FMM_OFF)
    s.set_option("solver", mfgb.SOLVER_CG)
    if args.pair_symmetric >= 0:
        s.set_option("pair_symmetric", args.pair_symmetric)
    if args.fused >= 0:
        s.set_option("fused_products", args.fused)
    s.solve(500)
    s.evaluate_fitted_near_foece()
    for _ in range(args.warmup):
        s.solve(500)
        s.evaluate_fitted_near_foece()
    s.set_option("kernel_timing", 1)
    s.reset_counters()
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    iters = []
    for _ in range(args.reps):
        iters.append(s.solve(500)[0])
        s.evaluate_fitted_near_foece()
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    out = {"kernel": args.kernel, "n": sc.n, "fused": s.get_option("fused_products"), "iters": iters}
    total = 0.0
    for kind, fpe in (("field", 49.0), ("force", 55.0), ("field_force", 86.0)):
        st = s.kernel_stats(kind)
        if st["launches"]:
            ms = st["total_ms"] / args.reps
            total += ms
            out[kind] = {"launches": st["launches"], "ms_per_step": ms,
                         "tflops": fpe * st["evals"] / (st["total_ms"] * 1e-3) / 1e12}
    out["pair_ms_per_step"] = total
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
