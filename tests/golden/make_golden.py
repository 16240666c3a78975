"""Generate tests/golden/golden_kernels.npz from the reference's own code.

Runs the reference's FMMTL pair kernels (DipoleBKernel, DipoleHessianKernel,
FP32, through fmmtl::direct) as compiled from the reference sources into
oracle/_ref/libmfref.so by oracle/Makefile.  Needs the reference sources, so
it runs only where they are mounted; the .npz it writes is committed and is
all the tests read.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as orc  # noqa: E402


def cases():
    rng = np.random.default_rng(20261203)
    out = {}
    # main.cu:7-35: 2x2x2 unit lattice, h = dx = 1, one external dipole (0,1,0)
    # at the origin (which coincides with a target), H0 = (0,1,0).
    g = np.array([[i, j, k] for i in range(2) for j in range(2) for k in range(2)], np.float32)
    out["grid8"] = dict(t=g, s=g, m=np.tile(np.float32([0, 1, 0]), (8, 1)), h=1.0)
    out["grid8_ext"] = dict(t=g, s=np.float32([[0, 0, 0]]), m=np.float32([[0, 1, 0]]), h=1.0)
    out["grid8_ext2"] = dict(t=g, s=np.float32([[0, -100, 0], [0, -101, 0]]), m=np.float32([[0, 1, 0], [0, 1, 0]]),
                             h=1.0)
    for n, h in ((1, 0.3), (2, 0.4), (3, 0.25), (31, 0.15), (64, 0.2), (513, 0.125)):
        x = rng.random((n, 3), dtype=np.float32)
        m = rng.normal(size=(n, 3)).astype(np.float32)
        out[f"rand{n}"] = dict(t=x, s=x, m=m, h=h)
    # pair distances on the branch boundaries of both kernels (q = r/h), along
    # generic directions and along +-z (the degenerate-frame case of
    # Dipole_hessian.kern:116)
    h = 0.5
    qs = np.float32([0.0, 0.25, 0.999, 1.0, 1.001, 1.5, 1.999, 2.0, 2.001, 2.5, 3.0, 3.5, 3.999, 4.0, 4.001, 5.0, 8.0])
    dirs = [np.float32([0, 0, 1]), np.float32([0, 0, -1]), np.float32([1, 0, 0]),
            np.float32([0.6, 0.0, 0.8]), np.float32([1, 2, 3]) / np.float32(np.sqrt(14.0))]
    t = []
    for q in qs:
        for d in dirs:
            t.append((q * h) * d)
    t = np.asarray(t, np.float32)
    out["boundary"] = dict(t=t, s=np.zeros((1, 3), np.float32), m=np.float32([[0.3, -0.5, 0.8]]), h=h)
    # targets / sources that differ (external-source shape), different h
    xt = rng.random((97, 3), dtype=np.float32)
    xs = rng.random((13, 3), dtype=np.float32) * 2 - 0.5
    ms = rng.normal(size=(13, 3)).astype(np.float32)
    out["ext97x13"] = dict(t=xt, s=xs, m=ms, h=0.3)
    return out


def main():
    orc.build(ref=True)
    ref = orc.RefKernels()
    blob = {}
    for name, c in cases().items():
        f = ref.field(c["t"], c["s"], c["m"], c["h"])
        T = ref.tensor(c["t"], c["s"], c["m"], c["h"])
        blob[f"{name}/targets"] = c["t"]
        blob[f"{name}/sources"] = c["s"]
        blob[f"{name}/charges"] = c["m"]
        blob[f"{name}/h"] = np.float32(c["h"])
        blob[f"{name}/field"] = f
        blob[f"{name}/tensor"] = T
    path = os.path.join(HERE, "golden_kernels.npz")
    np.savez_compressed(path, **blob)
    print(f"wrote {path} ({os.path.getsize(path)} bytes, {len(cases())} cases)")


if __name__ == "__main__":
    main()
