#!/usr/bin/env python
"""Pair interactions per second of the magnetization-and-force step on GB300.

Workload (default): N = 65,536 particles, jittered cubic lattice (jitter
+-0.25 spacing, seed 1) filling a sphere of radius 0.5, h = 2 x spacing,
chi = 2, H0 = (0,0,1), FP32 pair arithmetic with compensated accumulation,
FP64 solver inner products.  One step = one timestep: CG solve of the
magnetization (warm start, relative residual 1e-6), the Kelvin force, and a
symplectic Euler update with dt = 1e-4, all on the device.

Printed (rank 0, one JSON line):
  value      executed pair interactions (field + force) / device time, inputs
             resident in HBM; L2 flushed (256 MiB write) before every timed step
  e2e        the same metric through the public API with host buffers: every
             step uploads positions from pinned memory, solves, evaluates the
             force, reads M, B/mu0 and F back and integrates on the host
  roofline   FP32 FMA roofline of the dominant pair kernel: algorithmic FLOP
             (32 per ordered field pair, 53 per ordered force pair; for a
             product evaluated once per unordered pair, 49 / 55 per unordered
             pair) / its event-timed device time, against the FP32 peak
             SMs x 128 lanes x 2 FLOP x max SM clock (a dense-FFMA probe
             measured in this run is reported beside it)
  errors     M, B/mu0 and the Kelvin force of a cold solve of the same scene
             against the FP64 oracle's solution over all particles
             (tests/golden/config2_oracle.npz)
  batched_vs_plain, served_vs_plain
             the spec comparison: 256 scenes of 512..32,768 particles
             stepped in one launch per stage against the same scenes one at a
             time; a Poisson stream of scenes of 1,024..262,144 particles
             served with continuous batching against the same arrivals one
             request at a time (pairs/s and p50/p99 step and request latency)
  fmm_1048576  the 1,048,576-particle cylinder through the FMM (the fmm1m
             workload, a few steps): effective pairs/s, step latency, product
             times and the force's error against the FP64 oracle
  cpu_baseline  the CPU restatement of the reference's pair kernels (FP32,
             OpenMP over all host cores) on a bounded sample of the same step

``--impl reference`` times that CPU implementation alone (see run_reference).
Multi-GPU: one independent replica per rank (the step has no exchange), value
summed over ranks, time = max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "magnetic-force_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

FLOP_FIELD_PAIR = 32.0  # minimal far-field form, FMA = 2, rsqrt = 1
FLOP_FORCE_PAIR = 53.0
# one evaluation serving both particles of an unordered pair:
#   force: 49 FLOP for f_ij, plus 3 adds into the target and 3 into the source
#   field: 13 for d, r^2, rsqrt, r^-3, -3 r^-5; 10 for d.m_s and d.m_t; 2 for
#          their products with -3 r^-5; 2 x 3 x 2 FMA into each side's sum
FLOP_FORCE_UPAIR = 55.0
FLOP_FIELD_UPAIR = 49.0
# both products of the same dipoles in one evaluation (k_sym_ff): the field's
# 49 and the force's 55 less what they share, d 3, r^2 5, d.m_s 5, d.m_t 5
FLOP_FIELD_FORCE_UPAIR = 49.0 + 55.0 - 18.0


def product_flop(name, st):
    """Algorithmic FLOP of the timed launches of one product kind: the
    ordered pairs at the per-pair count, or, where one evaluation served both
    particles (evals < pairs), the unordered pairs at the per-evaluation count."""
    if name == "field_force":
        return FLOP_FIELD_FORCE_UPAIR * st["evals"], "k_sym_ff<field+force>"
    if st.get("evals", st["pairs"]) < st["pairs"]:
        return (FLOP_FORCE_UPAIR if name == "force" else FLOP_FIELD_UPAIR) * st["evals"], f"k_sym<{name}>"
    return (FLOP_FIELD_PAIR if name == "field" else FLOP_FORCE_PAIR) * st["pairs"], f"allpairs_kernel<{name}>"

# The FMA-pipe ceiling of each pair body: algorithmic FLOP per pipe cycle at a
# fully busy FMA pipe, against the peak's 2 FLOP per cycle (packed f32x2
# operations per target and pair item, counted from the bodies): the all-pairs
# field 19 per 2 ordered pairs (64 FLOP), force 30 (106 FLOP); once per
# unordered pair, field 30 per 2 unordered pairs (98 FLOP), force 36 (110 FLOP),
# both in one evaluation 54 (172 FLOP).
BODY_BOUND = {"allpairs_kernel<field>": 64.0 / 76.0, "allpairs_kernel<force>": 106.0 / 120.0,
              "k_sym<field>": 98.0 / 120.0, "k_sym<force>": 110.0 / 144.0,
              "k_sym_ff<field+force>": 2 * FLOP_FIELD_FORCE_UPAIR / 216.0}


def fp32_peak(sm_max_mhz):
    """Nominal FP32 FMA peak of device 0 in TFLOP/s: SMs x 128 FP32 lanes x 2
    FLOP per FMA x the maximum SM clock (nvidia-smi clocks.max.sm)."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = sm_max_mhz or 2070.0
    return sms * 128 * 2 * mhz * 1e6 / 1e12, sms, mhz


def pair_roofline(kf, kg, peak, n, probe=None, kff=None):
    """Roofline of the dominant pair product of a timed run from the handle's
    kernel statistics (field kf, force kg, both in one launch kff): per
    product its algorithmic TFLOP/s, fraction of the FP32 peak and of its
    body's ceiling."""
    kern = {}
    names = {}
    for name, st in (("field", kf), ("force", kg), ("field_force", kff or {"launches": 0})):
        if st["launches"]:
            flop, names[name] = product_flop(name, st)
            tflops = flop / (st["total_ms"] * 1e-3) / 1e12
            bound = BODY_BOUND.get(names[name])
            kern[name] = {"kernel": names[name], "launches": st["launches"], "total_ms": round(st["total_ms"], 4),
                          "avg_ms": round(st["total_ms"] / st["launches"], 4),
                          "pairs_per_launch": st["pairs"] / st["launches"],
                          "evals_per_launch": st["evals"] / st["launches"],
                          "flop_per_launch": flop / st["launches"],
                          "tflops": tflops, "frac": tflops / peak,
                          "body_bound": round(bound, 4) if bound else None,
                          "frac_of_body_bound": round(tflops / peak / bound, 4) if bound else None,
                          "pairs_per_s": st["pairs"] / (st["total_ms"] * 1e-3)}
            if name == "field_force":
                # the same launch at the two products' own counts (49 + 55 per
                # unordered pair), comparable with the separate k_sym launches
                t2 = (FLOP_FIELD_UPAIR + FLOP_FORCE_UPAIR) * st["evals"] / (st["total_ms"] * 1e-3) / 1e12
                kern[name]["tflops_at_product_counts"] = t2
                kern[name]["frac_at_product_counts"] = round(t2 / peak, 4)
    dom = max(kern, key=lambda k: kern[k]["total_ms"])
    ach = kern[dom]["tflops"]
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath) and n == 65536:
        key = f"sym_{dom}_fp32_65536" if names[dom].startswith("k_sym") else f"allpairs_{dom}_fp32_65536"
        traffic = json.load(open(tpath)).get(key)
    return {"bound": "fp32", "achieved": round(ach, 3), "peak": round(peak, 3), "unit": "TFLOP/s",
            "frac": round(ach / peak, 4), "traffic": traffic, "kernel": names[dom],
            "frac_of_body_bound": kern[dom]["frac_of_body_bound"],
            "peak_source": "SMs x 128 FP32 lanes x 2 FLOP x max SM clock (nvidia-smi clocks.max.sm)",
            "probe_tflops": round(probe, 3) if probe else None,
            "frac_of_probe": round(ach / probe, 4) if probe else None,
            "kernels": kern,
            "note": "pairwise sums are not a contraction: FP32 FMA pipe, not tensor cores. "
                    "Algorithmic FLOP: 32 per ordered field pair, 53 per ordered force pair; for a product "
                    "evaluated once per unordered pair (k_sym; its timed bracket includes the per-particle "
                    "finish) 49 (field) or 55 (force) per unordered pair, both in one evaluation (k_sym_ff) "
                    "86 (104 less the 18 the two share). frac_of_body_bound: frac over the "
                    "body's FMA-pipe ceiling (BODY_BOUND). DRAM traffic per launch: the 2 MB of pair-layout "
                    "records, read a few times (L2 absorbs the rest)"}

METRIC = "pair interactions/s; p50/p99 step latency, served vs plain at 1e-5 rel err"
UNIT = "pairs/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dt", type=float, default=1e-4)
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="served: skip the plain-path comparison")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--requests", type=int, default=24)
    ap.add_argument("--rate", type=float, default=0.0,
                    help="served: mean Poisson arrival rate, requests/s; 0 (default): 80 %% of the served "
                         "capacity measured first with every request arriving at once")
    ap.add_argument("--workload", default="allpairs65k",
                    choices=["allpairs65k", "batch256", "plain4096", "served", "fmm1m"],
                    help="allpairs65k: the headline config (default); batch256: 256 scenes log-uniform "
                         "in [512, 32768] in one launch per stage vs the same scenes one at a time; "
                         "plain4096: N=4096 uniform cube solved in FP64 to 1e-8; fmm1m: N=1,048,576 "
                         "jittered-lattice cylinder through the FMM (P=8, theta=0.5)")
    ap.add_argument("--fmm-order", type=int, default=8)
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--rel-tol", type=float, default=1e-6, help="CG relative residual tolerance of every solve")
    ap.add_argument("--no-compare", action="store_true",
                    help="default workload: skip the batched-vs-plain and served-vs-plain comparisons")
    ap.add_argument("--compare-steps", type=int, default=5,
                    help="default workload: timed batched timesteps of the batched-vs-plain comparison")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi sampled every 50 ms while the timed region runs.  start()
    returns once the sampler has written its first line; the lines written
    before that point are dropped, so the record covers the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None
        self.skip = 0

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
            return
        t_end = time.time() + 5.0
        while time.time() < t_end and self.proc.poll() is None:
            with open(self.path) as f:
                self.skip = sum(1 for _ in f)
            if self.skip:
                break
            time.sleep(0.01)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        rows = rows[self.skip:] if len(rows) > self.skip else rows[-1:]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_pair_rates(pos: np.ndarray, mom: np.ndarray, h: float, seconds: float):
    """FP32 CPU restatement of the reference's DipoleBKernel / DipoleHessianKernel
    (fmmtl::direct split over targets with OpenMP), timed on target chunks
    against all sources.  Returns (field pairs/s, force pairs/s, sample text)."""
    import oracle as orc
    o = orc.Oracle()
    n = len(pos)
    rates = {}
    done = {}
    for kind in ("field", "force"):
        budget = seconds / 2
        pairs = 0.0
        t_used = 0.0
        start = 0
        chunk = 1024 if kind == "field" else 256
        while t_used < budget:
            idx = np.arange(start, start + chunk) % n
            t0 = time.perf_counter()
            if kind == "field":
                o.field(pos[idx], pos, mom, h, prec=32)
            else:
                o.tensor_sum(pos[idx], pos, mom, h, prec=32)
            t_used += time.perf_counter() - t0
            pairs += chunk * n
            start += chunk
        rates[kind] = pairs / t_used
        done[kind] = (pairs, t_used)
    sample = (f"field: {int(done['field'][0] / n)} targets x {n} sources in {done['field'][1]:.1f} s; "
              f"force tensor: {int(done['force'][0] / n)} targets x {n} sources in {done['force'][1]:.1f} s")
    return rates["field"], rates["force"], sample


def run_ours(args, rank, world, local):
    import torch
    import mfgb
    import scenes

    torch.cuda.set_device(local)
    sc = scenes.config_allpairs_65k() if args.n == 65536 else scenes.jittered_lattice(args.n, "sphere", 0.5, chi=2.0)
    n = sc.n
    s = mfgb.Solver(n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos, device=local)
    s.set_option("solver", mfgb.SOLVER_CG)
    s.set_option("rel_tol", args.rel_tol)
    s.set_option("kernel_timing", 1)

    # cold solve (reported) + warm-up steps
    t0 = time.perf_counter()
    cold_iters, cold_res = s.solve(500)
    torch.cuda.synchronize()
    cold_ms = (time.perf_counter() - t0) * 1e3
    for _ in range(args.warmup):
        s.advance(args.dt, 500)
    torch.cuda.synchronize()

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > 129 MB L2
    s.reset_counters()
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    step_ms = []
    iters = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        iters.append(s.advance(args.dt, 500))
        e1.record()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ctr = s.counters()
    kf = s.kernel_stats("field")
    kg = s.kernel_stats("force")
    kff = s.kernel_stats("field_force")
    total_ms = sum(step_ms)
    pairs = ctr["field_pairs"] + ctr["force_pairs"]
    t_max = allreduce_max(total_ms, world)
    pairs_all = allreduce_sum(pairs, world)
    value = pairs_all / (t_max * 1e-3)

    # dominant pair kernel and its FP32 roofline
    peak, sms, mhz = fp32_peak(clk.get("sm_max_mhz"))
    roofline = pair_roofline(kf, kg, peak, n, probe=mfgb.probe_fp32_peak(), kff=kff)
    roofline["peak_inputs"] = {"sms": sms, "sm_max_mhz": mhz}

    # accuracy: a cold solve of the same scene against the FP64 oracle's
    # solution over all particles, and the final state's fixed-point residual
    # and force on a sample (FP64 oracle sums over all N)
    errors = None
    if rank == 0:
        errors = {"final_state_sample": sample_errors(s, sc)}
        if n == 65536:
            errors.update(config2_errors(args, local))

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(s, sc, args, world)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        M = s.M
        rf, rg, sample = cpu_pair_rates(sc.pos, M, sc.h, args.cpu_seconds)
        fp = ctr["field_pairs"]
        gp = ctr["force_pairs"]
        cpu_time = fp / rf + gp / rg
        cpu = {"value": (fp + gp) / cpu_time, "unit": UNIT, "cores": cpu_threads(), "kind": "port",
               "sample": sample + "; value = the timed step's field/force pair mix at these rates",
               "field_pairs_per_s": rf, "force_pairs_per_s": rg}
    s.close()

    # the spec comparison: batched and served against plain
    batched = served = fmm = None
    if not args.no_compare and n == 65536:
        batched = measure_batch(args, rank, world, local, steps=args.compare_steps, plain_passes=1)
        served = measure_served(args, rank, world, local)
        # config 3 (1,048,576 particles through the FMM), a few steps
        fs, _, _, fmm = fmm_measure(args, rank, world, local, steps=args.compare_steps, warmup=3)
        fs.close()

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded jittered-lattice sphere (the reference ships no dataset)",
            "config": config_allpairs(n, sc.h, args),
            "field_pairs": ctr["field_pairs"], "force_pairs": ctr["force_pairs"],
            "solve_iters_per_step": iters, "step_ms": [round(v, 4) for v in step_ms],
            "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
            "cold_solve": {"iters": cold_iters, "rel_res": cold_res, "ms": round(cold_ms, 3)},
            "gpu_launches": ctr["kernel_launches"],
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "errors": errors, "clocks": clk,
            "batched_vs_plain": summarize_batch(batched) if batched else None,
            "served_vs_plain": summarize_served(served) if served else None,
            "fmm_1048576": summarize_fmm(fmm) if fmm else None,
            "autotune": mfgb.autotune_report(),
        }
        print(json.dumps(out), flush=True)


def config_allpairs(n, h, args):
    """The default workload's config, shared by both arms of the bench."""
    return {"workload": f"allpairs_fp32_{n}: jittered lattice sphere r=0.5, N={n}, h=2*spacing={h:.5f}, chi=2, "
                        f"H0=(0,0,1), dt={args.dt}, CG rel tol {args.rel_tol:g}",
            "N": n, "step": "one timestep: warm-started CG solve + Kelvin force + symplectic Euler",
            "l2": "flushed before every timed step (256 MiB write, not timed)",
            "parallelism": f"replicas x{int(os.environ.get('WORLD_SIZE', '1'))}"}


def config2_errors(args, local):
    """A fresh handle at the fixture's positions (the same scene), solved cold
    to the bench's tolerance, its force evaluated: relative L2 of B/mu0, M and
    F over all particles against the FP64 oracle's solution, read from the
    committed fixture (oracle CG to a relative residual of 6e-12)."""
    import mfgb
    path = os.path.join(ROOT, "tests", "golden", "config2_oracle.npz")
    if not os.path.exists(path):
        return {"oracle_solution": "fixture missing"}
    z = np.load(path)
    pos = z["pos"]
    s = mfgb.Solver(len(pos), float(z["h"]), float(z["h"]), float(z["volume"]), float(z["chi"]), z["H0"], None,
                    None, pos, device=local)
    s.set_option("solver", mfgb.SOLVER_CG)
    s.set_option("rel_tol", args.rel_tol)
    it, rr = s.solve(500)
    s.evaluate_fitted_near_foece()
    c = float(z["volume"]) * float(z["chi"]) / (1.0 + float(z["chi"]))
    b = z["b"].astype(np.float64)
    rel = lambda a, w: float(np.linalg.norm(np.asarray(a, np.float64) - w) / np.linalg.norm(w))  # noqa: E731
    out = {"B_rel_l2": rel(s.total_B_over_mu0, b), "M_rel_l2": rel(s.M, c * b),
           "F_rel_l2": rel(s.magnetic_bodyforce, z["F"].astype(np.float64)),
           "over": f"all {len(pos)} particles x 3 components",
           "against": f"FP64 oracle CG solution (rel res {float(z['rel_res']):.1e}) and its Kelvin force "
                      "(tests/golden/config2_oracle.npz)",
           "solve": {"iters": int(it), "rel_res": float(rr), "rel_tol": args.rel_tol}}
    s.close()
    return out


def sample_errors(s, sc, k: int = 256):
    """Relative fixed-point residual |b - Hext - c G b| / |Hext| and force
    error on k sample particles, both with FP64 oracle sums over all N."""
    import oracle as orc
    o = orc.Oracle()
    rng = np.random.default_rng(0)
    idx = np.sort(rng.choice(sc.n, size=min(k, sc.n), replace=False))
    pos = s.xyz.astype(np.float64)
    b = s.get("total_B_over_mu0", f64=True)
    M = s.get("M", f64=True)
    Hext = s.get("Hext", f64=True)
    F = s.get("magnetic_bodyforce", f64=True)
    G = o.field(pos[idx], pos, M, sc.h)
    r = b[idx] - Hext[idx] - G
    T = o.tensor_sum(pos[idx], pos, M, sc.h).reshape(-1, 3, 3)  # [i][col][row]
    Fo = np.einsum("icr,ic->ir", T, M[idx])
    return {"sample": int(len(idx)),
            "fixed_point_rel_residual": float(np.linalg.norm(r) / np.linalg.norm(Hext[idx])),
            "force_rel_l2": float(np.linalg.norm(F[idx] - Fo) / np.linalg.norm(Fo))}


def run_e2e(s, sc, args, world):
    import torch
    n = sc.n
    pin = lambda: torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()  # noqa: E731
    pos, F, B, M = pin(), pin(), pin(), pin()
    pos[:] = s.xyz
    vel = np.zeros((n, 3), np.float32)
    s.reset_counters()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.setTargetpos(pos)                 # H2D
        s.solve(500)
        s.evaluate_fitted_near_foece()
        s.get("magnetic_bodyforce", out=F)  # D2H
        s.get("total_B_over_mu0", out=B)
        s.get("M", out=M)
        vel += np.float32(args.dt) * F / np.float32(sc.volume)
        pos += np.float32(args.dt) * vel
    torch.cuda.synchronize()
    dt_s = time.perf_counter() - t0
    ctr = s.counters()
    dt_max = allreduce_max(dt_s, world)
    pairs = allreduce_sum(ctr["field_pairs"] + ctr["force_pairs"], world)
    return {"value": pairs / dt_max, "unit": UNIT, "h2d_bytes_per_step": n * 12, "d2h_bytes_per_step": 3 * n * 12,
            "ms_per_step": dt_max * 1e3 / args.steps, "path": "mf_set_positions/mf_solve/mf_eval_force/mf_get"}


def run_reference(args, rank, world):
    """The reference's CPU path for this step: its pair kernels evaluated all-
    pairs on the host (the CPU restatement, FP32, OpenMP over every core).
    The reference sources are not present where this runs, so the port stands
    in for them (the port is bit-identical to the reference's FP32 field
    kernel and within 2e-6 on the force tensor, pinned by tests/test_oracle.py).
    Same scene, metric and config as the GPU arm, and the same work mix: the
    GPU's timed step evaluates one field product and one force product over
    all N^2 pairs, so each CPU step is a bounded sample of both, the same
    number of targets for each (1:1), against all N sources, with the
    dipoles of the solved magnetization (M = c b of the FP64 oracle's
    solution of this scene, tests/golden/config2_oracle.npz); value =
    executed pairs / wall time."""
    if rank != 0:
        return
    import oracle as orc
    import scenes
    sc = scenes.config_allpairs_65k() if args.n == 65536 else scenes.jittered_lattice(args.n, "sphere", 0.5, chi=2.0)
    o = orc.Oracle()
    n = sc.n
    path = os.path.join(ROOT, "tests", "golden", "config2_oracle.npz")
    if n == 65536 and os.path.exists(path):
        z = np.load(path)
        pos = np.ascontiguousarray(z["pos"], np.float32)
        mom = (sc.c * z["b"].astype(np.float64)).astype(np.float32)
        dipoles = "M = c b of the FP64 oracle's solution of this scene"
    else:
        pos = sc.pos
        rng = np.random.default_rng(1)
        mom = ((np.array([0.0, 0.0, 1.0]) + 0.1 * rng.normal(size=(n, 3))) * sc.c).astype(np.float32)
        dipoles = "seeded moments c (H0 + 0.1 N(0,1))"
    nt = 256

    def step(k):
        i0 = (k * nt) % n
        idx = np.arange(i0, i0 + nt) % n
        o.field(pos[idx], pos, mom, sc.h, prec=32)
        o.tensor_sum(pos[idx], pos, mom, sc.h, prec=32)
        return 2 * nt * n

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    pairs = 0.0
    for k in range(args.steps):
        pairs += step(args.warmup + k)
    dt = time.perf_counter() - t0
    value = pairs / dt
    cores = cpu_threads()
    sample = (f"{nt} field targets + {nt} force-tensor targets x {n} sources per step (the GPU step's 1:1 "
              f"field:force pair mix), {dipoles}, FP32, OpenMP {cores} threads")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
           "data": "synthetic: seeded jittered-lattice sphere (the reference ships no dataset)",
           "config": config_allpairs(n, sc.h, args),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def measure_batch(args, rank, world, local, steps, plain_passes):
    """Batched scenes (one launch per stage for all, graph-captured timesteps)
    against the plain path (each scene through its own solver, one after the
    other), same scenes, kernels, tolerance and step.  Returns the record."""
    import torch
    import mfgb
    import scenes

    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    scs = scenes.batched_scenes(args.scenes, seed=7 + 1000 * rank)
    gen_s = time.perf_counter() - t0
    n_tot = sum(s.n for s in scs)
    b = mfgb.Batch(scs, device=local)
    cold_it, cold_res = b.solve(500, args.rel_tol)
    b.advance(args.dt, max(3, args.warmup), iters_per_step=4, rel_tol=args.rel_tol, graph=True)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    b.reset_counters()
    clocks = ClockSampler(local)
    barrier(world)
    clocks.start()
    step_ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        b.advance(args.dt, 1, iters_per_step=4, rel_tol=args.rel_tol, graph=True)
        step_ms.append((time.perf_counter() - t) * 1e3)
    barrier(world)
    clk = clocks.stop()
    c = b.counters()
    rr, its = b.solver_state()
    pairs = c["field_pairs"] + c["force_pairs"]
    total_ms = sum(step_ms)
    t_max = allreduce_max(total_ms, world)
    value = allreduce_sum(pairs, world) / (t_max * 1e-3)
    b.close()

    # plain path: the same scenes one at a time through the single-scene solver
    solvers = []
    for sc in scs:
        s = mfgb.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos, device=local)
        s.set_option("solver", mfgb.SOLVER_CG)
        s.set_option("rel_tol", args.rel_tol)
        s.solve(500)
        s.advance(args.dt, 500)
        s.reset_counters()
        solvers.append(s)
    torch.cuda.synchronize()
    plain_ms = 0.0
    plain_pairs = 0.0
    plain_steps = []
    for _ in range(plain_passes):
        t_pass = 0.0
        for s in solvers:
            flush.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            s.advance(args.dt, 4)
            torch.cuda.synchronize()
            t_pass += (time.perf_counter() - t) * 1e3
        plain_steps.append(t_pass)
        plain_ms += t_pass
    for s in solvers:
        cc = s.counters()
        plain_pairs += cc["field_pairs"] + cc["force_pairs"]
        s.close()
    plain_value = plain_pairs / (plain_ms * 1e-3)
    return {
        "value": value, "ms_per_step": t_max / steps, "steps": steps,
        "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
        "step_ms": [round(v, 3) for v in step_ms],
        "field_pairs": c["field_pairs"], "force_pairs": c["force_pairs"], "gpu_launches": c["kernel_launches"],
        "cold_solve": {"max_iters": cold_it, "worst_rel_res": cold_res},
        "worst_rel_res_last_step": float(np.max(rr)), "max_iters_last_step": float(np.max(its)),
        "plain": {"value": plain_value, "unit": UNIT, "ms_per_step": plain_ms / plain_passes,
                  "passes": plain_passes, "path": "one mf_solver per scene, scenes one after the other, "
                                                  "L2 flushed before each scene's step"},
        "batched_over_plain": value / plain_value,
        "scenes": len(scs), "particles": n_tot, "scene_generation_s": round(gen_s, 1), "clocks": clk,
        "config": {"workload": f"batch{len(scs)}: {len(scs)} scenes, N log-uniform in [512, 32768] "
                               f"(total {n_tot}), radius U(0.2,0.5), chi U(0.5,3), H0 random unit, dt={args.dt}, "
                               f"CG rel tol {args.rel_tol:g}, <= 4 CG iterations per step, one CUDA graph per "
                               "timestep", "scenes": len(scs), "particles": n_tot,
                   "l2": "flushed before every timed step (256 MiB write, not timed)"},
    }


def summarize_batch(r):
    """The batched-vs-plain comparison as carried on the default line."""
    return {"batched": {"value": r["value"], "unit": UNIT, "ms_per_step": r["ms_per_step"],
                        "p50_step_ms": r["p50_step_ms"], "p99_step_ms": r["p99_step_ms"], "steps": r["steps"],
                        "gpu_launches": r["gpu_launches"], "max_iters_last_step": r["max_iters_last_step"]},
            "plain": {"value": r["plain"]["value"], "unit": UNIT, "ms_per_step": r["plain"]["ms_per_step"],
                      "passes": r["plain"]["passes"]},
            "ratio": r["batched_over_plain"], "config": r["config"], "clocks": r["clocks"]}


def run_batch(args, rank, world, local):
    import mfgb
    r = measure_batch(args, rank, world, local, steps=args.steps, plain_passes=max(1, min(args.steps, 3)))
    if rank == 0:
        out = {
            "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded jittered-lattice spheres (the reference ships no dataset)",
            "config": r["config"],
            "autotune": mfgb.autotune_report(),
        }
        out.update({k: v for k, v in r.items() if k not in ("value", "ms_per_step", "config", "steps")})
        print(json.dumps(out), flush=True)


def run_plain_fp64(args, rank, world, local):
    """N=4096 uniform cube, V=(1/16)^3, h=2V^(1/3), chi=1, H0=(0,0,1): FP64
    solve to 1e-8 relative residual and one force pass, checked against the
    FP64 oracle."""
    import torch
    import mfgb
    import oracle as orc
    import scenes

    torch.cuda.set_device(local)
    sc = scenes.config_plain_fp64()
    times = []
    for k in range(args.warmup + args.steps):
        # a fresh solver per step (untimed) so every timed solve starts cold
        s = mfgb.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos, precision="fp64",
                        device=local)
        s.set_option("solver", mfgb.SOLVER_CG)
        s.set_option("rel_tol", 1e-8)
        torch.cuda.synchronize()
        t = time.perf_counter()
        it, rr = s.solve(500)
        s.evaluate_fitted_near_foece()
        torch.cuda.synchronize()
        if k >= args.warmup:
            times.append((time.perf_counter() - t) * 1e3)
        if k + 1 < args.warmup + args.steps:
            s.close()
    o = orc.Oracle()
    hext, _ = o.ext(sc.pos, None, None, sc.H0, sc.h)
    b, _, _ = o.solve_cg(sc.pos, sc.h, sc.c, hext, rel_tol=1e-13)
    F = o.force(sc.pos, sc.c * b, sc.h)
    rel = lambda a, w: float(np.linalg.norm(a - w) / np.linalg.norm(w))  # noqa: E731
    c = s.counters()
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload": "plain4096_fp64", "ms_per_step_median": float(np.median(times)),
                          "cg_iters": it, "rel_res": rr,
                          "errors_vs_fp64_oracle": {"B": rel(s.get("total_B_over_mu0", f64=True), b),
                                                    "M": rel(s.get("M", f64=True), sc.c * b),
                                                    "F": rel(s.get("magnetic_bodyforce", f64=True), F)}}), flush=True)
    s.close()


def served_requests(args, rank):
    """The served stream's requests (seeded): N log-uniform in [1024, 262144],
    the batched config's per-scene distributions."""
    import math
    import scenes
    rng = np.random.default_rng(99 + rank)
    reqs = []
    for k in range(args.requests):
        n = int(round(math.exp(rng.uniform(math.log(1024), math.log(262144)))))
        r2 = np.random.default_rng(5000 + k)
        H = r2.normal(size=3)
        H /= np.linalg.norm(H)
        reqs.append(scenes.jittered_lattice(n, "sphere", radius=float(r2.uniform(0.2, 0.5)),
                                            chi=float(r2.uniform(0.5, 3.0)), seed=5000 + k, H0=tuple(H)))
    gaps = rng.exponential(1.0, size=len(reqs))  # unit-rate Poisson gaps, scaled by the rate
    return reqs, gaps


def measure_served(args, rank, world, local):
    """Served stream: Poisson arrivals (seeded) of scenes with N log-uniform
    in [1024, 262144] and the batched config's per-scene distributions, 20
    timesteps each, continuous batching under a 120 GB budget.  Scenes up to
    65,536 particles join the all-pairs batch; larger ones run as their own
    solver handle (field products through the FMM, the force as the handle's
    automatic choice picks it), each on its own host thread and stream beside
    the batch.  The mean rate is --rate, or by default 80 % of the served
    capacity, measured first by submitting every request at once.  Pairs are
    executed pairs for batch members and effective pairs (N^2 per product) for
    FMM products.  Reports p50/p99 per step, per tick and per request and
    aggregate pairs/s, beside the plain path on the same arrivals
    (run_served_plain)."""
    import torch
    import mfgb
    import scenes

    torch.cuda.set_device(local)
    reqs, gaps = served_requests(args, rank)
    capacity = None
    if args.rate <= 0:
        # Capacity: every request submitted at once, served to the last one.
        srv = mfgb.Server(hbm_budget_bytes=120e9, max_active=64, steps_per_request=20, iters_per_step=4,
                          rel_tol=args.rel_tol, dt=args.dt, device=local)
        t0 = time.perf_counter()
        cids = [srv.submit(r) for r in reqs]
        while any(srv.poll(i)[0] != 2 for i in cids):
            srv.step()
        capacity = len(reqs) / (time.perf_counter() - t0)
        srv.close()
        rate = 0.8 * capacity
    else:
        rate = args.rate
    arrivals = np.cumsum(gaps / rate)
    srv = mfgb.Server(hbm_budget_bytes=120e9, max_active=64, steps_per_request=20, iters_per_step=4,
                      rel_tol=args.rel_tol, dt=args.dt, device=local)
    # warm-up request (kernel load, first allocations), not measured
    wid = srv.submit(scenes.jittered_lattice(2048, "sphere", 0.3, chi=1.0, seed=1))
    while srv.poll(wid)[0] != 2:
        srv.step()
    s0 = srv.stats()
    ids = []
    tick_ms = []
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    while len(ids) < len(reqs) or any(srv.poll(i)[0] != 2 for i in ids):
        now = time.perf_counter() - t0
        while len(ids) < len(reqs) and arrivals[len(ids)] <= now:
            ids.append(srv.submit(reqs[len(ids)]))
        st = srv.stats()
        if st["running"] + st["queued"] > 0:
            a, c, ms = srv.step()
            if srv.stats()["ticks"] > st["ticks"]:  # the batch took a timestep
                tick_ms.append(ms)
        else:
            time.sleep(max(0.0, min(0.05, arrivals[len(ids)] - now)))
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    s1 = srv.stats()
    pairs = (s1["field_pairs"] + s1["force_pairs"]) - (s0["field_pairs"] + s0["force_pairs"])
    lat = [srv.poll(i)[2] for i in ids]
    big = [k for k, r in enumerate(reqs) if r.n > 65536]
    steps_all = np.concatenate([srv.step_times(i) for i in ids])
    steps_fmm = np.concatenate([srv.step_times(ids[k]) for k in big]) if big else np.zeros(0)
    steps_batch = np.concatenate([srv.step_times(ids[k]) for k in range(len(reqs)) if k not in big])
    pct = lambda v, q: float(np.percentile(v, q)) if len(v) else None  # noqa: E731
    srv.close()
    plain = run_served_plain(reqs, arrivals, args, local) if (rank == 0 and not args.no_plain) else None
    ns = [r.n for r in reqs]
    return {
        "value": pairs / wall, "unit": UNIT,
        "requests": len(reqs), "rate_per_s": rate,
        "rate_basis": ("80 % of the measured served capacity" if capacity else "given"),
        "capacity_req_per_s": capacity, "n_range": [min(ns), max(ns)], "n_mean": float(np.mean(ns)),
        "wall_s": wall, "busy_s": (s1["busy_ms"] - s0["busy_ms"]) / 1e3,
        "p50_step_ms": pct(steps_all, 50), "p99_step_ms": pct(steps_all, 99),
        "step_ms_by_path": {"batch": {"steps": len(steps_batch), "p50": pct(steps_batch, 50),
                                      "p99": pct(steps_batch, 99)},
                            "fmm": {"steps": len(steps_fmm), "p50": pct(steps_fmm, 50), "p99": pct(steps_fmm, 99)}},
        "p50_tick_ms": float(np.percentile(tick_ms, 50)) if tick_ms else None,
        "p99_tick_ms": float(np.percentile(tick_ms, 99)) if tick_ms else None,
        "p50_request_ms": float(np.percentile(lat, 50)), "p99_request_ms": float(np.percentile(lat, 99)),
        "ticks": s1["ticks"] - s0["ticks"], "rebatches": s1["rebatches"] - s0["rebatches"],
        "pairs": pairs, "budget_bytes": 120e9, "clocks": clk, "plain": plain,
        "note": "N <= 65,536: all-pairs batch (executed pairs); N > 65,536: own solver handle on its own host "
                "thread and stream, field products through the FMM (P=8, effective pairs), the force all-pairs "
                "up to 90,000 particles and through the FMM above; 20 timesteps per request, <= 4 CG "
                "iterations per step; step latency: per request timestep (batch members: their tick until the "
                "step was done on the device; others: each timestep on their thread); tick: serving-loop "
                "ticks in which the batch took a timestep",
    }


def summarize_served(r):
    """The served-vs-plain comparison as carried on the default line."""
    keys = ("value", "unit", "p50_step_ms", "p99_step_ms", "p50_request_ms", "p99_request_ms")
    out = {"served": {k: r[k] for k in keys}, "plain": None, "ratio": None,
           "requests": r["requests"], "rate_per_s": r["rate_per_s"], "rate_basis": r["rate_basis"],
           "capacity_req_per_s": r["capacity_req_per_s"], "n_range": r["n_range"],
           "p50_tick_ms": r["p50_tick_ms"], "p99_tick_ms": r["p99_tick_ms"],
           "step_ms_by_path": r["step_ms_by_path"], "clocks": r["clocks"], "note": r["note"]}
    if r["plain"]:
        out["plain"] = {k: r["plain"][k] for k in keys}
        out["plain"]["capacity_req_per_s"] = r["plain"]["capacity_req_per_s"]
        out["ratio"] = r["value"] / r["plain"]["value"]
        if r["capacity_req_per_s"]:
            out["capacity_ratio"] = r["capacity_req_per_s"] / r["plain"]["capacity_req_per_s"]
    return out


def run_served(args, rank, world, local):
    r = measure_served(args, rank, world, local)
    if rank == 0:
        out = {"metric": METRIC, "workload": "served"}
        out.update(r)
        print(json.dumps(out), flush=True)


def run_served_plain(reqs, arrivals, args, local):
    """The plain path on the served stream: the same requests, in arrival
    order, one at a time through their own solver handle (the same automatic
    choice of FMM or all-pairs per product as the served requests, CG to the
    same tolerance, the same 20 timesteps of <= 4 iterations).  Each request's
    service time (handle creation, cold solve, timesteps, read-back) is
    measured on the GPU; the queue is replayed on those times with the served
    run's arrival times (a request starts when it has arrived and the previous
    one is done).  Handles of every request are created once beforehand, so
    the autotuner's first timings (cached per process) are not charged to the
    plain path."""
    import torch
    import mfgb

    for sc in reqs:
        mfgb.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos, device=local).close()
    step_ms, lat_ms = [], []
    pairs = 0.0
    busy = 0.0
    done_at = 0.0
    t_first = float(arrivals[0])
    for k, sc in enumerate(reqs):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s = mfgb.Solver(sc.n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos, device=local)
        s.set_option("solver", mfgb.SOLVER_CG)
        s.set_option("rel_tol", args.rel_tol)
        s.solve(500)
        for _ in range(20):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            s.advance(args.dt, 4)
            torch.cuda.synchronize()
            step_ms.append((time.perf_counter() - t1) * 1e3)
        s.get("magnetic_bodyforce")
        c = s.counters()
        pairs += c["field_pairs"] + c["force_pairs"]
        s.close()
        service = time.perf_counter() - t0
        busy += service
        start = max(float(arrivals[k]), done_at)
        done_at = start + service
        lat_ms.append((done_at - float(arrivals[k])) * 1e3)
    makespan = done_at - t_first
    return {"value": pairs / makespan, "unit": UNIT, "makespan_s": makespan, "busy_s": busy,
            "capacity_req_per_s": len(reqs) / busy,
            "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
            "p50_request_ms": float(np.percentile(lat_ms, 50)), "p99_request_ms": float(np.percentile(lat_ms, 99)),
            "path": "one solver handle per request, requests one after the other in arrival order; queue "
                    "replayed on the measured service times"}


FMM_FORCE_ORDER, FMM_FORCE_THETA = 10, 0.44  # the handle's defaults for the Kelvin force products


def fmm_measure(args, rank, world, local, steps, warmup, n=1 << 20):
    """Config 3 on one GPU: N = 1,048,576 jittered-lattice cylinder (r = 0.3,
    height 1, h = 2 spacings, chi = 1.5, H0 = (0,0,1)) through the FMM: field
    products at P = 8 and theta 0.5, the Kelvin force at its own P = 10 and
    theta 0.44 (the handle's defaults), leaf boxes of >= 12 particles on
    average.  A step is one timestep as in the headline workload; effective
    pairs count N^2 per product (the FMM convention).  Returns the handle (still
    open), the scene and the measured summary; errors are sampled on rank 0
    against the FP64 oracle at 2,048 seeded targets (CPU)."""
    import torch
    import mfgb
    import scenes

    torch.cuda.set_device(local)
    sc = scenes.config_fmm_1m(n)
    n = sc.n
    s = mfgb.Solver(n, sc.h, sc.h, sc.volume, sc.chi, sc.H0, None, None, sc.pos, device=local)
    s.set_option("solver", mfgb.SOLVER_CG)
    s.set_option("rel_tol", args.rel_tol)
    s.set_option("fmm", mfgb.FMM_ON)
    s.set_option("fmm_order", args.fmm_order)
    s.set_option("fmm_theta", 0.5)
    s.set_option("kernel_timing", 1)
    t0 = time.perf_counter()
    cold_iters, cold_res = s.solve(500)
    torch.cuda.synchronize()
    cold_ms = (time.perf_counter() - t0) * 1e3
    for _ in range(warmup):
        s.advance(args.dt, 500)
    torch.cuda.synchronize()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    s.reset_counters()
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    step_ms, iters = [], []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        iters.append(s.advance(args.dt, 500))
        e1.record()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    del flush
    ctr = s.counters()
    st = s.fmm_stats()
    ks = {k: s.kernel_stats(k) for k in ("field", "force", "fmm_near_field", "fmm_near_force", "fmm_far")}
    total_ms = sum(step_ms)
    t_max = allreduce_max(total_ms, world)
    pairs = allreduce_sum(ctr["field_pairs"] + ctr["force_pairs"], world)
    value = pairs / (t_max * 1e-3)
    executed = st["field_products"] * st["p2p_pairs"] + st["force_products"] * st["force_p2p_pairs"]

    peak, _, _ = fp32_peak(clk.get("sm_max_mhz"))
    probe = mfgb.probe_fp32_peak()
    kern = {}
    for name, fpp, fpu in (("fmm_near_field", FLOP_FIELD_PAIR, FLOP_FIELD_UPAIR),
                           ("fmm_near_force", FLOP_FORCE_PAIR, FLOP_FORCE_UPAIR)):
        k = ks[name]
        if k["launches"]:
            # once per unordered box pair (evals < pairs): the per-evaluation count
            flop = fpu * k["evals"] if k["evals"] < k["pairs"] else fpp * k["pairs"]
            kern[name] = {"launches": k["launches"], "total_ms": round(k["total_ms"], 4),
                          "avg_ms": round(k["total_ms"] / k["launches"], 4),
                          "pairs_per_launch": k["pairs"] / k["launches"],
                          "evals_per_launch": k["evals"] / k["launches"],
                          "once_per_box_pair": k["evals"] < k["pairs"],
                          "tflops": flop / (k["total_ms"] * 1e-3) / 1e12}
    far = ks["fmm_far"]
    dom = max(kern, key=lambda k: kern[k]["total_ms"])
    roofline = {"bound": "fp32", "achieved": round(kern[dom]["tflops"], 3), "peak": round(peak, 3),
                "unit": "TFLOP/s", "frac": round(kern[dom]["tflops"] / peak, 4), "traffic": None,
                "kernel": ("k_fmm_near_sym + k_fmm_p2p<force>" if kern[dom].get("once_per_box_pair")
                           else f"k_fmm_p2p<{'force' if dom.endswith('force') else 'field'}>"),
                "peak_source": "SMs x 128 FP32 lanes x 2 FLOP x max SM clock (nvidia-smi clocks.max.sm)",
                "probe_tflops": round(probe, 3),
                "kernels": kern,
                "far_field": {"launches": far["launches"], "total_ms": round(far["total_ms"], 4),
                              "m2l_per_product": st["m2l_per_product"],
                              "force_m2l_per_product": st["force_m2l_per_product"]},
                "products_ms": {"field": ks["field"]["total_ms"] / max(ks["field"]["launches"], 1),
                                "force": ks["force"]["total_ms"] / max(ks["force"]["launches"], 1)},
                "note": "near-field kernels: executed pairs x minimal far-form FLOP (32 field, 53 force), or, "
                        "for the force's near field once per unordered box pair (k_fmm_near_sym + the read-back "
                        "in k_fmm_p2p), its evaluations x 55, / their event-timed duration"}
    errors = None
    if rank == 0:
        errors = sample_errors(s, sc, k=2048)
        errors["oracle"] = "FP64 CPU oracle sums over all N at 2,048 seeded targets"
    summary = {
        "metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": t_max / steps,
        "config": {"workload": f"fmm_fp32_{n}: jittered lattice cylinder r=0.3 height 1, N={n}, "
                               f"h=2*spacing={sc.h:.5f}, chi=1.5, H0=(0,0,1), FMM field P={args.fmm_order} "
                               f"theta=0.5, force P={FMM_FORCE_ORDER} theta={FMM_FORCE_THETA}, leaf>=12, "
                               f"dt={args.dt}, CG rel tol {args.rel_tol:g}",
                   "N": n, "step": "one timestep: octree rebuild, warm-started CG solve (FMM products), "
                                   "Kelvin force (FMM), symplectic Euler",
                   "l2": "flushed before every timed step (256 MiB write, not timed)",
                   "parallelism": f"replicas x{world}", "pairs": "effective (N^2 per product)"},
        "field_pairs": ctr["field_pairs"], "force_pairs": ctr["force_pairs"],
        "executed_near_pairs": executed, "fmm": st,
        "solve_iters_per_step": iters, "step_ms": [round(v, 4) for v in step_ms],
        "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
        "cold_solve": {"iters": cold_iters, "rel_res": cold_res, "ms": round(cold_ms, 3)},
        "gpu_launches": ctr["kernel_launches"], "roofline": roofline, "errors": errors, "clocks": clk,
    }
    return s, sc, ctr, summary


def run_fmm(args, rank, world, local):
    """The fmm1m workload (config 3) as its own line: fmm_measure plus a
    65,536-target check against the FP32 all-pairs direct kernels, the
    end-to-end rate and the CPU baseline."""
    import torch
    import mfgb

    s, sc, ctr, out = fmm_measure(args, rank, world, local, args.steps, args.warmup,
                                  n=args.n if args.n != 65536 else 1 << 20)
    n = sc.n
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath) and n == 1 << 20:
        dom = out["roofline"]["kernel"]
        key = ("fmm_near_sym_force" if "near_sym" in dom else "fmm_p2p_force" if "force" in dom
               else "fmm_p2p_field")
        out["roofline"]["traffic"] = json.load(open(tpath)).get(f"{key}_fp32_{n}")
    if rank == 0:
        # 65,536 seeded targets against the FP32 all-pairs direct kernels
        rng = np.random.default_rng(65536)
        idx = np.sort(rng.choice(n, size=min(65536, n), replace=False))
        pos = torch.from_numpy(s.xyz).cuda()
        M = torch.from_numpy(s.M).cuda()
        b = s.total_B_over_mu0[idx].astype(np.float64)
        hext = s.Hext[idx].astype(np.float64)
        G = mfgb.direct_field(pos[idx], pos, M, sc.h).double().cpu().numpy()
        r = b - hext - G  # fixed point b = Hext + G(c b), with M = c b
        T = mfgb.direct_force_tensor(pos[idx], pos, M, sc.h).double().cpu().numpy().reshape(-1, 3, 3)
        Fd = np.einsum("icr,ic->ir", T, M[idx].double().cpu().numpy())
        F = s.magnetic_bodyforce[idx].astype(np.float64)
        out["errors"]["subsample_65536"] = {
            "fixed_point_rel_residual": float(np.linalg.norm(r) / np.linalg.norm(hext)),
            "force_rel_l2": float(np.linalg.norm(F - Fd) / np.linalg.norm(Fd)),
            "against": "FP32 all-pairs direct kernels (mf_direct_field / mf_direct_force_tensor)"}
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(s, sc, args, world)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rf, rg, sample = cpu_pair_rates(sc.pos, s.M, sc.h, args.cpu_seconds)
        cpu_time = ctr["field_pairs"] / rf + ctr["force_pairs"] / rg
        cpu = {"value": (ctr["field_pairs"] + ctr["force_pairs"]) / cpu_time, "unit": UNIT,
               "cores": cpu_threads(), "kind": "port",
               "sample": sample + "; value = the timed step's effective field/force pairs at these direct rates "
                                  "(the CPU evaluates them all-pairs)"}
    if rank == 0:
        line = {"metric": METRIC, "value": out["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": out["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic: seeded jittered-lattice cylinder (the reference ships no dataset)"}
        line.update({k: v for k, v in out.items() if k not in line})
        line["cpu_baseline"] = cpu
        line["e2e"] = e2e
        print(json.dumps(line), flush=True)
    s.close()


def summarize_fmm(out):
    """The config-3 figures carried in the default line."""
    r = out["roofline"]
    e = out["errors"] or {}
    return {"workload": out["config"]["workload"], "value": out["value"], "unit": out["unit"],
            "ms_per_step": out["ms_per_step"], "p50_step_ms": out["p50_step_ms"], "p99_step_ms": out["p99_step_ms"],
            "products_ms": r["products_ms"], "executed_near_pairs": out["executed_near_pairs"],
            "roofline": {k: r[k] for k in ("kernel", "achieved", "peak", "unit", "frac")},
            "errors": {k: e.get(k) for k in ("fixed_point_rel_residual", "force_rel_l2", "oracle", "sample")},
            "solve_iters_per_step": out["solve_iters_per_step"], "clocks": out["clocks"]}


def main():
    args = parse()
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "served":
        run_served(args, rank, world, local)
    elif args.workload == "batch256":
        run_batch(args, rank, world, local)
    elif args.workload == "plain4096":
        run_plain_fp64(args, rank, world, local)
    elif args.workload == "fmm1m":
        run_fmm(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
