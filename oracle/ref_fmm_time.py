"""TEST INFRASTRUCTURE: times the reference's own CPU FMM (oracle/_ref/libmfref_fmm.so,
built by oracle/Makefile where the reference sources are present) on the FMM
workloads' shapes, and measures its error against the FP64 oracle.

The reference's sources exist only where they are mounted, so this runs there
(never on a machine that runs the GPU bench); its printed JSON lines are the
figures quoted for the reference's FMM.

    python oracle/ref_fmm_time.py --n 1048576 --order 8
    python oracle/ref_fmm_time.py --n 262144 --order 6

Per product kind (field, Hessian): the set-up and first product (tree,
interaction lists, plan), one further product on the same plan, and the
relative L2 error at seeded targets against FP64 direct sums over all N, with
the magnetization M = c (H0 + 0.3 N(0, 1)) on the config-3 cylinder (r = 0.3,
height 1, h = 2 spacings, chi = 1.5).  The force is F_i = T_i m_i.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "magnetic-force_gb300"))
import oracle as orc  # noqa: E402
import scenes  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--order", type=int, default=8)
    ap.add_argument("--ncrit", type=int, default=384)
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--targets", type=int, default=1024)
    args = ap.parse_args()
    orc.build(ref=True)
    ref = orc.RefFmm()
    o = orc.Oracle()
    sc = scenes.config_fmm_1m(args.n)
    rng = np.random.default_rng(1)
    m = ((np.array([0.0, 0.0, 1.0]) + 0.3 * rng.normal(size=(sc.n, 3))) * sc.c).astype(np.float32)
    idx = np.sort(rng.choice(sc.n, min(args.targets, sc.n), replace=False))
    p64, m64 = sc.pos.astype(np.float64), m.astype(np.float64)
    threads = len(os.sched_getaffinity(0))
    for kind in ("field", "hessian"):
        fn = ref.field if kind == "field" else ref.hessian
        out, first, per = fn(sc.pos, m, sc.h, order=args.order, ncrit=args.ncrit, theta=args.theta, reps=1)
        t0 = time.time()
        if kind == "field":
            want = o.field(p64[idx], p64, m64, sc.h)
            err = np.linalg.norm(out[idx] - want) / np.linalg.norm(want)
        else:
            T = o.tensor_sum(p64[idx], p64, m64, sc.h).reshape(-1, 3, 3)
            want = np.einsum("icr,ic->ir", T, m64[idx])
            got = np.einsum("icr,ic->ir", out[idx].astype(np.float64).reshape(-1, 3, 3), m64[idx])
            err = np.linalg.norm(got - want) / np.linalg.norm(want)
        print(json.dumps({"kind": kind, "n": sc.n, "order": args.order, "ncrit": args.ncrit, "theta": args.theta,
                          "setup_and_first_product_s": round(first, 3), "product_s": round(per, 3),
                          "effective_pairs_per_s": float(sc.n) ** 2 / per if per > 0 else None,
                          "rel_l2_error": float(err), "error_targets": int(len(idx)),
                          "error_of": "B/mu0" if kind == "field" else "Kelvin force T_i m_i",
                          "host_threads": threads, "oracle_s": round(time.time() - t0, 1)}), flush=True)


if __name__ == "__main__":
    main()
