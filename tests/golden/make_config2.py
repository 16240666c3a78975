"""Generate tests/golden/config2_oracle.npz: the FP64 oracle's solution of the
65,536-particle all-pairs scene (jittered-lattice sphere r = 0.5, h = 2
spacings, chi = 2, H0 = (0, 0, 1); scenes.config_allpairs_65k()).

The CPU oracle (oracle/mf_oracle.c) solves (I - c G) b = Hext by FP64 CG to
a relative residual of 1e-11 over all N (magnetic_force.cu:1016-1017 define
the residual, c = V chi / (1 + chi)), then evaluates the Kelvin force at
M = c b over every particle (magnetic_force.cu:583-603).  The full solve is
~20 all-pairs FP64 products of 4.3e9 pairs each -- minutes on a few host
cores -- so it is computed once here and committed; the GPU tests and the
bench read the file.

Stored (float32 is ample for comparisons at 1e-5: 6e-8 relative):
  pos  [N, 3] float32  the scene's positions (used as given, not regenerated)
  b    [N, 3] float32  B/mu0 of the FP64 solve
  F    [N, 3] float32  Kelvin force at M = c b
  h, volume, chi, H0, iters, rel_res

    python tests/golden/make_config2.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "magnetic-force_gb300"))
import oracle as orc  # noqa: E402
import scenes  # noqa: E402


def main():
    orc.build(ref=False)
    o = orc.Oracle()
    sc = scenes.config_allpairs_65k()
    pos = np.ascontiguousarray(sc.pos, np.float32)
    p64 = pos.astype(np.float64)
    c = sc.volume * sc.chi / (1.0 + sc.chi)
    hext, _ = o.ext(p64, None, None, sc.H0, sc.h)
    t0 = time.time()
    b, iters, rr = o.solve_cg(p64, sc.h, c, hext, rel_tol=1e-11, max_iter=200)
    t1 = time.time()
    F = o.force(p64, c * b, sc.h)
    t2 = time.time()
    path = os.path.join(HERE, "config2_oracle.npz")
    np.savez_compressed(path, pos=pos, b=b.astype(np.float32), F=F.astype(np.float32), h=np.float64(sc.h),
                        volume=np.float64(sc.volume), chi=np.float64(sc.chi), H0=np.asarray(sc.H0, np.float64),
                        iters=np.int64(iters), rel_res=np.float64(rr))
    print(f"wrote {path} ({os.path.getsize(path)} bytes): N={len(pos)} CG iters={iters} rel_res={rr:.2e} "
          f"solve {t1 - t0:.0f} s, force {t2 - t1:.0f} s")


if __name__ == "__main__":
    main()
