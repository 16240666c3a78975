"""TEST INFRASTRUCTURE: ctypes loader for the CPU oracle (libmforacle.so) and,
where it was built, the reference's own FMMTL pair kernels (_ref/libmfref.so).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module; the shipped library never does.

All arrays are numpy, AoS ``[n, 3]`` for positions / moments / fields and
``[n, 9]`` (glm column-major, ``T[c*3 + r]``) for force tensors.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "libmforacle.so")
_REF = os.path.join(HERE, "_ref", "libmfref.so")

_i64 = ctypes.c_int64
_p = ctypes.c_void_p


def build(ref: bool = True) -> None:
    """Compile the oracle (and oracle/_ref when the reference sources exist)."""
    target = "all" if ref else "oracle"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Oracle:
    """FP64 restatement (``*_f64``) plus the same arithmetic in FP32 (``*_f32``)."""

    def __init__(self, path: str = _LIB):
        if not os.path.exists(path):
            build(ref=False)
        self.lib = ctypes.CDLL(path)
        for sfx in ("_f64", "_f32"):
            for name in ("orc_field", "orc_tensor_sum"):
                f = getattr(self.lib, name + sfx)
                f.restype = None
            f = getattr(self.lib, "orc_force" + sfx)
            f.restype = None
            f = getattr(self.lib, "orc_ext" + sfx)
            f.restype = None
            f = getattr(self.lib, "orc_pair_field" + sfx)
            f.restype = None
            f = getattr(self.lib, "orc_pair_force_tensor" + sfx)
            f.restype = None
        self.lib.orc_solve_nlcg.restype = ctypes.c_int
        self.lib.orc_solve_cg.restype = ctypes.c_int

    @staticmethod
    def _dt(prec):
        return (np.float64, "_f64", ctypes.c_double) if prec == 64 else (np.float32, "_f32", ctypes.c_float)

    def _arr(self, a, dt, cols=3):
        a = np.ascontiguousarray(np.asarray(a, dtype=dt).reshape(-1, cols))
        return a

    # -- pair kernels ------------------------------------------------------
    def pair_field(self, d, m, h, prec=64):
        dt, sfx, cr = self._dt(prec)
        d = np.ascontiguousarray(d, dtype=dt)
        m = np.ascontiguousarray(m, dtype=dt)
        out = np.zeros(3, dtype=dt)
        getattr(self.lib, "orc_pair_field" + sfx)(_p(_ptr(d)), _p(_ptr(m)), cr(h), _p(_ptr(out)))
        return out

    def pair_force_tensor(self, d, s, h, prec=64):
        dt, sfx, cr = self._dt(prec)
        d = np.ascontiguousarray(d, dtype=dt)
        s = np.ascontiguousarray(s, dtype=dt)
        out = np.zeros(9, dtype=dt)
        getattr(self.lib, "orc_pair_force_tensor" + sfx)(_p(_ptr(d)), _p(_ptr(s)), cr(h), _p(_ptr(out)))
        return out

    # -- all-pairs sums ----------------------------------------------------
    def field(self, tpos, spos, smom, h, prec=64):
        """B/mu0 at targets from dipoles (fmmtl::direct over DipoleBKernel)."""
        dt, sfx, cr = self._dt(prec)
        t, s, m = self._arr(tpos, dt), self._arr(spos, dt), self._arr(smom, dt)
        out = np.zeros_like(t)
        getattr(self.lib, "orc_field" + sfx)(_i64(len(t)), _p(_ptr(t)), _i64(len(s)), _p(_ptr(s)),
                                             _p(_ptr(m)), cr(h), _p(_ptr(out)))
        return out

    def tensor_sum(self, tpos, spos, smom, h, prec=64):
        dt, sfx, cr = self._dt(prec)
        t, s, m = self._arr(tpos, dt), self._arr(spos, dt), self._arr(smom, dt)
        out = np.zeros((len(t), 9), dtype=dt)
        getattr(self.lib, "orc_tensor_sum" + sfx)(_i64(len(t)), _p(_ptr(t)), _i64(len(s)), _p(_ptr(s)),
                                                  _p(_ptr(m)), cr(h), _p(_ptr(out)))
        return out

    def force(self, pos, mom, h, rext=None, naive_quirks=False, prec=64):
        dt, sfx, cr = self._dt(prec)
        x, m = self._arr(pos, dt), self._arr(mom, dt)
        out = np.zeros_like(x)
        rp = None
        if rext is not None:
            rext = self._arr(rext, dt, 9)
            rp = _p(_ptr(rext))
        getattr(self.lib, "orc_force" + sfx)(_i64(len(x)), _p(_ptr(x)), _p(_ptr(m)), cr(h), rp,
                                             ctypes.c_int(1 if naive_quirks else 0), _p(_ptr(out)))
        return out

    def ext(self, pos, spos, smom, H0, hs, prec=64):
        dt, sfx, cr = self._dt(prec)
        x = self._arr(pos, dt)
        if spos is None or len(spos) == 0:
            s = np.zeros((0, 3), dtype=dt)
            m = np.zeros((0, 3), dtype=dt)
        else:
            s, m = self._arr(spos, dt), self._arr(smom, dt)
        H = np.ascontiguousarray(H0, dtype=dt)
        hext = np.zeros_like(x)
        rext = np.zeros((len(x), 9), dtype=dt)
        getattr(self.lib, "orc_ext" + sfx)(_i64(len(x)), _p(_ptr(x)), _i64(len(s)), _p(_ptr(s) if len(s) else 0),
                                           _p(_ptr(m) if len(m) else 0), _p(_ptr(H)), cr(hs),
                                           _p(_ptr(hext)), _p(_ptr(rext)))
        return hext, rext

    # -- solvers (FP64) ----------------------------------------------------
    def solve_nlcg(self, pos, h, volume, chi, hext, b0=None, tolerance=0.1, niter=100, max_iteration=80):
        x = self._arr(pos, np.float64)
        he = self._arr(hext, np.float64)
        b = np.zeros_like(x) if b0 is None else self._arr(b0, np.float64).copy()
        errs = np.zeros(int(min(niter, max_iteration)) + 4, dtype=np.float64)
        ne = ctypes.c_int64(0)
        steps = self.lib.orc_solve_nlcg(_i64(len(x)), _p(_ptr(x)), ctypes.c_double(h), ctypes.c_double(volume),
                                        ctypes.c_double(chi), _p(_ptr(he)), _p(_ptr(b)),
                                        ctypes.c_double(tolerance), _i64(niter), _i64(max_iteration),
                                        _p(_ptr(errs)), ctypes.byref(ne))
        return b, errs[: ne.value].copy(), steps

    def solve_cg(self, pos, h, c, hext, b0=None, rel_tol=1e-12, max_iter=1000):
        x = self._arr(pos, np.float64)
        he = self._arr(hext, np.float64)
        b = np.zeros_like(x) if b0 is None else self._arr(b0, np.float64).copy()
        rr = ctypes.c_double(0)
        it = self.lib.orc_solve_cg(_i64(len(x)), _p(_ptr(x)), ctypes.c_double(h), ctypes.c_double(c),
                                   _p(_ptr(he)), _p(_ptr(b)), ctypes.c_double(rel_tol), ctypes.c_int(max_iter),
                                   ctypes.byref(rr))
        return b, it, rr.value


class RefFmm:
    """The reference's own CPU FMM (fmmtl::kernel_matrix, FP64 spherical
    expansions, OpenMP), built from its sources into _ref/libmfref_fmm.so."""

    PATH = os.path.join(HERE, "_ref", "libmfref_fmm.so")

    def __init__(self, path: str = PATH):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        for f in (self.lib.ref_fmm_field, self.lib.ref_fmm_hessian):
            f.restype = ctypes.c_int
            f.argtypes = [_i64, _p, _p, ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                          _p, _p]

    @staticmethod
    def available(path: str = PATH) -> bool:
        return os.path.exists(path)

    def _run(self, fn, cols, pos, mom, h, order, ncrit, theta, reps):
        x = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        m = np.ascontiguousarray(mom, dtype=np.float32).reshape(-1, 3)
        out = np.zeros((len(x), cols), np.float32)
        sec = np.zeros(2, np.float64)
        fn(_i64(len(x)), _p(_ptr(x)), _p(_ptr(m)), ctypes.c_float(h), int(order), int(ncrit), float(theta),
           int(reps), _p(_ptr(out)), _p(_ptr(sec)))
        return out, float(sec[0]), float(sec[1])

    def field(self, pos, mom, h, order=6, ncrit=384, theta=0.5, reps=0):
        """B/mu0 at every particle; returns (result, set-up + first product s, s per further product)."""
        return self._run(self.lib.ref_fmm_field, 3, pos, mom, h, order, ncrit, theta, reps)

    def hessian(self, pos, mom, h, order=6, ncrit=384, theta=0.5, reps=0):
        """The force tensors [n][9] (glm column-major) at every particle."""
        return self._run(self.lib.ref_fmm_hessian, 9, pos, mom, h, order, ncrit, theta, reps)


class RefKernels:
    """The reference's own FMMTL kernels (FP32), built from its sources."""

    def __init__(self, path: str = _REF):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        self.lib.ref_field.restype = ctypes.c_int
        self.lib.ref_tensor.restype = ctypes.c_int

    @staticmethod
    def available(path: str = _REF) -> bool:
        return os.path.exists(path)

    def field(self, tpos, spos, smom, h):
        t = np.ascontiguousarray(tpos, dtype=np.float32).reshape(-1, 3)
        s = np.ascontiguousarray(spos, dtype=np.float32).reshape(-1, 3)
        m = np.ascontiguousarray(smom, dtype=np.float32).reshape(-1, 3)
        out = np.zeros_like(t)
        self.lib.ref_field(_i64(len(t)), _p(_ptr(t)), _i64(len(s)), _p(_ptr(s)), _p(_ptr(m)),
                           ctypes.c_float(h), _p(_ptr(out)))
        return out

    def tensor(self, tpos, spos, smom, h):
        t = np.ascontiguousarray(tpos, dtype=np.float32).reshape(-1, 3)
        s = np.ascontiguousarray(spos, dtype=np.float32).reshape(-1, 3)
        m = np.ascontiguousarray(smom, dtype=np.float32).reshape(-1, 3)
        out = np.zeros((len(t), 9), dtype=np.float32)
        self.lib.ref_tensor(_i64(len(t)), _p(_ptr(t)), _i64(len(s)), _p(_ptr(s)), _p(_ptr(m)),
                            ctypes.c_float(h), _p(_ptr(out)))
        return out
