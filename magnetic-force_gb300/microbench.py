"""Kernel-level timing of the all-pairs launches (also the small case used for
Nsight Compute captures).

    python magnetic-force_gb300/microbench.py --kernel field --n 65536 --reps 5

Runs mf_direct_field / mf_direct_force / mf_direct_force_tensor on a seeded
jittered-lattice sphere of N particles (h = 2 x spacing) with random dipoles,
times each launch with CUDA events and prints one JSON line per kernel:
device ms per call (packing included), pairs/s and algorithmic TFLOP/s.
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
    ap.add_argument("--kernel", default="field", choices=["field", "force", "tensor", "all"])
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    args = ap.parse_args()

    import numpy as np
    import torch

    import mfgb
    import scenes

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
        for _ in range(args.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            call()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        best = min(times)
        pairs = float(sc.n) * sc.n
        print(json.dumps({"kernel": kind, "n": sc.n, "ms_best": best, "ms_all": times,
                          "pairs_per_s": pairs / (best * 1e-3),
                          "tflops": FLOP[kind] * pairs / (best * 1e-3) / 1e12}), flush=True)


if __name__ == "__main__":
    main()
