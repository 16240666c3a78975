"""Seeded synthetic particle clouds for tests and benchmarks.

The reference ships no datasets or benchmark inputs; these generators stand
in for them with the shapes and parameters of the benchmark configurations:

* ``uniform_cube``  N points uniform in [0,1]^3 (the plain FP64 case, N=4096,
  V=(1/16)^3, h=2 V^(1/3)).
* ``jittered_lattice``  a cubic lattice with spacing s, each point jittered by
  U(-0.25 s, 0.25 s)^3, clipped to a shape (sphere or cylinder); s is bisected
  until at least N points fall inside, then the points farthest from the
  centroid are dropped so exactly N remain.  Particle volume V = V_shape / N,
  smoothing length h = 2 s.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Scene:
    pos: np.ndarray          # [N, 3] float32
    h: float
    volume: float
    chi: float
    H0: tuple = (0.0, 0.0, 1.0)
    spacing: float = 0.0
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.pos)

    @property
    def c(self) -> float:
        return self.volume * self.chi / (1.0 + self.chi)


def uniform_cube(n: int = 4096, seed: int = 1, volume: float = (1 / 16) ** 3, chi: float = 1.0,
                 H0=(0.0, 0.0, 1.0)) -> Scene:
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 3)).astype(np.float32)
    return Scene(pos=pos, h=2.0 * volume ** (1.0 / 3.0), volume=volume, chi=chi, H0=tuple(H0),
                 meta={"shape": "cube", "seed": seed})


def _inside(shape: str, p: np.ndarray, radius: float, height: float) -> np.ndarray:
    if shape == "sphere":
        return np.einsum("ij,ij->i", p, p) <= radius * radius
    if shape == "cylinder":
        return (p[:, 0] ** 2 + p[:, 1] ** 2 <= radius * radius) & (np.abs(p[:, 2]) <= 0.5 * height)
    raise ValueError(shape)


def _shape_volume(shape: str, radius: float, height: float) -> float:
    if shape == "sphere":
        return 4.0 / 3.0 * math.pi * radius ** 3
    return math.pi * radius * radius * height


def _lattice(shape: str, s: float, radius: float, height: float, seed: int) -> np.ndarray:
    ext = np.array([radius, radius, radius if shape == "sphere" else 0.5 * height])
    k = np.ceil(ext / s).astype(int) + 1
    axes = [np.arange(-kk, kk + 1, dtype=np.float64) * s for kk in k]
    g = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    g = g + rng.uniform(-0.25 * s, 0.25 * s, size=g.shape)
    return g[_inside(shape, g, radius, height)]


def jittered_lattice(n: int, shape: str = "sphere", radius: float = 0.5, height: float = 1.0, chi: float = 2.0,
                     seed: int = 1, H0=(0.0, 0.0, 1.0)) -> Scene:
    vs = _shape_volume(shape, radius, height)
    s0 = (vs / n) ** (1.0 / 3.0)
    lo, hi = 0.7 * s0, 1.3 * s0  # count(lo) >= n > count(hi)
    while len(_lattice(shape, lo, radius, height, seed)) < n:
        lo *= 0.9
    while len(_lattice(shape, hi, radius, height, seed)) >= n:
        hi *= 1.1
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        if len(_lattice(shape, mid, radius, height, seed)) >= n:
            lo = mid
        else:
            hi = mid
    s = lo
    pts = _lattice(shape, s, radius, height, seed)
    if len(pts) > n:
        cen = pts.mean(axis=0)
        d = np.einsum("ij,ij->i", pts - cen, pts - cen)
        keep = np.sort(np.argsort(d, kind="stable")[:n])
        pts = pts[keep]
    assert len(pts) == n
    return Scene(pos=pts.astype(np.float32), h=2.0 * s, volume=vs / n, chi=chi, H0=tuple(H0), spacing=s,
                 meta={"shape": shape, "radius": radius, "height": height, "seed": seed})


def config_plain_fp64() -> Scene:
    """N=4096 uniform in the unit cube, V=(1/16)^3, h=2V^(1/3), chi=1, H0=(0,0,1)."""
    return uniform_cube(4096, seed=1, volume=(1 / 16) ** 3, chi=1.0)


def config_allpairs_65k() -> Scene:
    """N=65,536 jittered lattice in a sphere of radius 0.5, h=2 s, chi=2, H0=(0,0,1)."""
    return jittered_lattice(65536, "sphere", radius=0.5, chi=2.0, seed=1)


def config_fmm_1m(n: int = 1 << 20) -> Scene:
    """N=1,048,576 jittered-lattice cylinder r=0.3, height 1, chi=1.5."""
    return jittered_lattice(n, "cylinder", radius=0.3, height=1.0, chi=1.5, seed=1)


def batched_scenes(count: int = 256, lo: int = 512, hi: int = 32768, seed: int = 7) -> list[Scene]:
    """Independent scenes, N log-uniform in [lo, hi], sphere radius U(0.2, 0.5),
    chi U(0.5, 3.0), H0 a random unit vector; scene i uses seed + i."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        radius = float(rng.uniform(0.2, 0.5))
        chi = float(rng.uniform(0.5, 3.0))
        H = rng.normal(size=3)
        H /= np.linalg.norm(H)
        sc = jittered_lattice(n, "sphere", radius=radius, chi=chi, seed=seed + i, H0=tuple(float(v) for v in H))
        out.append(sc)
    return out
