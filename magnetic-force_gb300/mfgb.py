"""Python host binding of libmfgb.so (include/mf.h) over ctypes.

``Solver`` mirrors the reference's ``Libo::cuda_magnet_cgOptimizer``
(magnetic_solver/magnetic_force.cuh:36-174): the same constructor arguments,
the same method names (``setTargetpos``, ``setHext``, ``solve``,
``evaluate_fitted_near_foece``, ``export_data``, ``export_force``) and the
same public results (``M``, ``total_B_over_mu0``, ``Hext``,
``magnetic_bodyforce``, ``dHextdx/dy/dz``), returned here as numpy arrays
of shape [n, 3].  Knobs ``tolerance``, ``max_iteration`` and ``naive`` are
properties, as they are public members in the reference.

``direct_field`` / ``direct_force_tensor`` / ``direct_force`` evaluate the
reference's FMMTL pair kernels all-pairs on device buffers (torch CUDA
tensors), the replacement of ``fmmtl::direct``.

There is no CPU fallback: if the library or a CUDA device is missing the
calls raise.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmfgb.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "mf.h")

MF_OK = 0
STATUS = {
    0: "MF_OK", 1: "MF_ERR_INVALID_ARG", 2: "MF_ERR_OOM", 3: "MF_ERR_NOT_CONVERGED", 4: "MF_ERR_CUDA",
    5: "MF_ERR_TIMEOUT", 6: "MF_ERR_BUDGET", 7: "MF_ERR_UNSUPPORTED", 8: "MF_ERR_BUSY",
}
LAYOUT_AOS, LAYOUT_SOA = 0, 1
HOST, DEVICE = 0, 1
FP32, FP64 = 0, 1
Q = {"positions": 0, "M": 1, "total_B_over_mu0": 2, "Hext": 3, "magnetic_bodyforce": 4,
     "dHextdx": 5, "dHextdy": 6, "dHextdz": 7, "velocity": 8}
OPT = {"tolerance": 0, "max_iteration": 1, "naive": 2, "solver": 3, "rel_tol": 4, "cg_max_iter": 5,
       "crit_size": 6, "check_interval": 7, "kernel_timing": 8, "fmm": 9, "fmm_order": 10, "fmm_theta": 11,
       "fmm_leaf": 12, "autotune": 13, "pair_symmetric": 14, "fmm_force_theta": 15,
       "fmm_force_order": 16, "fused_products": 17}
FMM_AUTO, FMM_ON, FMM_OFF = 0, 1, 2
SOLVER_NLCG, SOLVER_CG = 0, 1


class MFError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class mf_params(ctypes.Structure):
    _fields_ = [
        ("num_particles", ctypes.c_int64), ("h", ctypes.c_float), ("ext_mag_h", ctypes.c_float),
        ("volume", ctypes.c_float), ("chi", ctypes.c_float), ("const_ext_field", ctypes.c_float * 3),
        ("target_pos", ctypes.c_void_p), ("ext_source_pos", ctypes.c_void_p), ("ext_source_M", ctypes.c_void_p),
        ("n_ext", ctypes.c_int64), ("precision", ctypes.c_int32), ("device", ctypes.c_int32),
    ]


class mf_counters(ctypes.Structure):
    _fields_ = [("field_products", ctypes.c_int64), ("force_passes", ctypes.c_int64),
                ("field_pairs", ctypes.c_double), ("force_pairs", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64)]


class mf_kernel_stats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_int64), ("total_ms", ctypes.c_double), ("pairs", ctypes.c_double),
                ("evals", ctypes.c_double)]


class mf_fmm_stats(ctypes.Structure):
    _fields_ = [("active", ctypes.c_int32), ("levels", ctypes.c_int32), ("leaf_level", ctypes.c_int32),
                ("degree", ctypes.c_int32), ("leaf_boxes", ctypes.c_int64), ("occupied_leaves", ctypes.c_int64),
                ("max_leaf", ctypes.c_int32), ("near_rows", ctypes.c_int32), ("p2p_pairs", ctypes.c_double),
                ("m2l_per_product", ctypes.c_double), ("launches_per_product", ctypes.c_int32),
                ("force_active", ctypes.c_int32), ("field_products", ctypes.c_int64),
                ("force_products", ctypes.c_int64), ("theta", ctypes.c_double), ("force_theta", ctypes.c_double),
                ("force_p2p_pairs", ctypes.c_double), ("force_m2l_per_product", ctypes.c_double)]


KERNEL = {"field": 0, "force": 1, "tensor": 2, "fmm_near_field": 3, "fmm_near_force": 4, "fmm_far": 5,
          "field_force": 6}

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libmfgb.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: build it with magnetic-force_gb300/build.py")
    lib = ctypes.CDLL(path)
    i32, i64, vp, f32, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_float, ctypes.c_double
    sig = {
        "mf_status_string": (ctypes.c_char_p, [i32]),
        "mf_last_error": (ctypes.c_char_p, []),
        "mf_abi_version": (ctypes.c_int, []),
        "mf_create": (i32, [ctypes.POINTER(mf_params), ctypes.POINTER(vp)]),
        "mf_destroy": (i32, [vp]),
        "mf_set_stream": (i32, [vp, vp]),
        "mf_set_positions": (i32, [vp, vp, i64, i32, i32]),
        "mf_set_external": (i32, [vp, vp, vp, vp, i64, f32]),
        "mf_solve": (i32, [vp, i64, ctypes.POINTER(i64), ctypes.POINTER(f64)]),
        "mf_get_error_history": (i32, [vp, vp, i64, ctypes.POINTER(i64)]),
        "mf_eval_force": (i32, [vp]),
        "mf_get": (i32, [vp, i32, vp, i32, i32]),
        "mf_get_f64": (i32, [vp, i32, vp, i32, i32]),
        "mf_device_soa": (i32, [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]),
        "mf_num_particles": (i32, [vp, ctypes.POINTER(i64)]),
        "mf_set_option": (i32, [vp, i32, f64]),
        "mf_get_option": (i32, [vp, i32, ctypes.POINTER(f64)]),
        "mf_export_data": (i32, [vp, ctypes.c_char_p]),
        "mf_export_force": (i32, [vp, ctypes.c_char_p]),
        "mf_advance": (i32, [vp, f64, i64, ctypes.POINTER(i64)]),
        "mf_get_counters": (i32, [vp, ctypes.POINTER(mf_counters)]),
        "mf_reset_counters": (i32, [vp]),
        "mf_direct_field": (i32, [vp, i64, vp, vp, i64, f32, vp, vp]),
        "mf_direct_force_tensor": (i32, [vp, i64, vp, vp, i64, f32, vp, vp]),
        "mf_direct_force": (i32, [vp, vp, i64, f32, vp, i32, vp, vp]),
        "mf_release_scratch": (i32, []),
        "mf_debug_stage_wait_limit": (i32, [i64]),
        "mf_get_kernel_stats": (i32, [vp, i32, ctypes.POINTER(mf_kernel_stats)]),
        "mf_probe_fp32_peak": (i32, [ctypes.POINTER(f64)]),
        "mf_get_fmm_stats": (i32, [vp, ctypes.POINTER(mf_fmm_stats)]),
        "mf_apply_field": (i32, [vp, vp, i32, i32, vp]),
        "mf_autotune_report": (i32, [vp, i64, ctypes.POINTER(i64)]),
        "mf_fmm_create": (i32, [vp, i64, vp, i64, f32, i32, f64, i32, i32, ctypes.POINTER(vp)]),
        "mf_fmm_destroy": (i32, [vp]),
        "mf_fmm_field": (i32, [vp, vp, vp]),
        "mf_fmm_hessian": (i32, [vp, vp, vp]),
        "mf_fmm_get_stats": (i32, [vp, ctypes.POINTER(mf_fmm_stats)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def declared_symbols(header: str = HEADER) -> list[str]:
    """Function names declared in include/*.h (for the export check)."""
    names = set()
    hdir = os.path.dirname(header)
    for fn in sorted(os.listdir(hdir)):
        if fn.endswith(".h"):
            txt = open(os.path.join(hdir, fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names.update(re.findall(r"\b(mf_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def check(status: int) -> None:
    if status != MF_OK:
        msg = load().mf_last_error()
        raise MFError(status, msg.decode() if msg else "")


def _f32(a, cols=3) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, cols))


class Solver:
    """``Libo::cuda_magnet_cgOptimizer`` on libmfgb.so."""

    def __init__(self, num_particles, h, ext_mag_h, volume, chi, const_ext_field, ext_source_pos,
                 ext_source_M, target_pos, precision: str = "fp32", device: int = 0):
        lib = load()
        tp = _f32(target_pos)
        if len(tp) != num_particles:
            raise ValueError("target_pos does not have num_particles rows")
        esp = _f32(ext_source_pos) if ext_source_pos is not None and len(ext_source_pos) else np.zeros((0, 3), np.float32)
        esm = _f32(ext_source_M) if ext_source_M is not None and len(ext_source_M) else np.zeros((0, 3), np.float32)
        p = mf_params()
        p.num_particles = int(num_particles)
        p.h, p.ext_mag_h, p.volume, p.chi = float(h), float(ext_mag_h), float(volume), float(chi)
        for k in range(3):
            p.const_ext_field[k] = float(const_ext_field[k])
        p.target_pos = tp.ctypes.data
        p.ext_source_pos = esp.ctypes.data if len(esp) else None
        p.ext_source_M = esm.ctypes.data if len(esm) else None
        p.n_ext = len(esp)
        p.precision = FP64 if precision == "fp64" else FP32
        p.device = int(device)
        self._keep = (tp, esp, esm)
        h_ = ctypes.c_void_p()
        check(lib.mf_create(ctypes.byref(p), ctypes.byref(h_)))
        self._h = h_
        self.precision = precision

    def close(self):
        if getattr(self, "_h", None):
            load().mf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- methods of the reference class -------------------------------------
    def setTargetpos(self, pos):
        a = _f32(pos)
        check(load().mf_set_positions(self._h, a.ctypes.data, len(a), LAYOUT_AOS, HOST))

    def set_positions_device(self, ptr: int, n: int, layout: int = LAYOUT_AOS):
        check(load().mf_set_positions(self._h, ctypes.c_void_p(ptr), n, layout, DEVICE))

    def setHext(self, const_ext_field, ext_source_pos, ext_source_M, ext_mag_h):
        H = np.ascontiguousarray(const_ext_field, dtype=np.float32)
        sp = _f32(ext_source_pos) if ext_source_pos is not None and len(ext_source_pos) else np.zeros((0, 3), np.float32)
        sm = _f32(ext_source_M) if ext_source_M is not None and len(ext_source_M) else np.zeros((0, 3), np.float32)
        check(load().mf_set_external(self._h, H.ctypes.data, sp.ctypes.data if len(sp) else None,
                                     sm.ctypes.data if len(sm) else None, len(sp), float(ext_mag_h)))

    def solve(self, niter: int = 100):
        it = ctypes.c_int64(0)
        err = ctypes.c_double(0)
        st = load().mf_solve(self._h, int(niter), ctypes.byref(it), ctypes.byref(err))
        if st not in (MF_OK, 3):
            check(st)
        self.last_status = st
        return it.value, err.value

    def evaluate_fitted_near_foece(self):
        check(load().mf_eval_force(self._h))

    def advance(self, dt: float, niter: int = 100) -> int:
        it = ctypes.c_int64(0)
        st = load().mf_advance(self._h, float(dt), int(niter), ctypes.byref(it))
        if st not in (MF_OK, 3):
            check(st)
        return it.value

    def export_data(self, path: str):
        check(load().mf_export_data(self._h, path.encode()))

    def export_force(self, path: str):
        check(load().mf_export_force(self._h, path.encode()))

    def set_stream(self, stream_ptr: int):
        check(load().mf_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    # -- results ---------------------------------------------------------------
    @property
    def np(self) -> int:
        n = ctypes.c_int64(0)
        check(load().mf_num_particles(self._h, ctypes.byref(n)))
        return n.value

    def get(self, quantity: str, f64: bool = False, out: np.ndarray | None = None) -> np.ndarray:
        n = self.np
        if out is None:
            out = np.empty((n, 3), dtype=np.float64 if f64 else np.float32)
        assert out.flags["C_CONTIGUOUS"] and out.size == 3 * n
        assert out.dtype == (np.float64 if f64 else np.float32)
        fn = load().mf_get_f64 if f64 else load().mf_get
        check(fn(self._h, Q[quantity], out.ctypes.data, LAYOUT_AOS, HOST))
        return out

    def get_into_device(self, quantity: str, ptr: int, f64: bool = False, layout: int = LAYOUT_AOS):
        fn = load().mf_get_f64 if f64 else load().mf_get
        check(fn(self._h, Q[quantity], ctypes.c_void_p(ptr), layout, DEVICE))

    def device_soa(self, quantity: str):
        x, y, z = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check(load().mf_device_soa(self._h, Q[quantity], ctypes.byref(x), ctypes.byref(y), ctypes.byref(z)))
        return x.value, y.value, z.value

    def error_history(self) -> np.ndarray:
        n = ctypes.c_int64(0)
        check(load().mf_get_error_history(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float64)
        check(load().mf_get_error_history(self._h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def counters(self) -> dict:
        c = mf_counters()
        check(load().mf_get_counters(self._h, ctypes.byref(c)))
        return {f: getattr(c, f) for f, _ in mf_counters._fields_}

    def reset_counters(self):
        check(load().mf_reset_counters(self._h))

    def kernel_stats(self, kind: str) -> dict:
        st = mf_kernel_stats()
        check(load().mf_get_kernel_stats(self._h, KERNEL[kind], ctypes.byref(st)))
        return {"launches": st.launches, "total_ms": st.total_ms, "pairs": st.pairs, "evals": st.evals}

    def fmm_stats(self) -> dict:
        st = mf_fmm_stats()
        check(load().mf_get_fmm_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in mf_fmm_stats._fields_}

    def apply_field(self, moments) -> np.ndarray:
        """G(m) at the particles: the reference's cuda_magnet_cgOptimizer::G."""
        m = _f32(moments)
        out = np.empty_like(m)
        check(load().mf_apply_field(self._h, m.ctypes.data, LAYOUT_AOS, HOST, out.ctypes.data))
        return out

    def set_option(self, key: str, value: float):
        check(load().mf_set_option(self._h, OPT[key], float(value)))

    def get_option(self, key: str) -> float:
        v = ctypes.c_double(0)
        check(load().mf_get_option(self._h, OPT[key], ctypes.byref(v)))
        return v.value

    M = property(lambda self: self.get("M"))
    total_B_over_mu0 = property(lambda self: self.get("total_B_over_mu0"))
    Hext = property(lambda self: self.get("Hext"))
    magnetic_bodyforce = property(lambda self: self.get("magnetic_bodyforce"))
    dHextdx = property(lambda self: self.get("dHextdx"))
    dHextdy = property(lambda self: self.get("dHextdy"))
    dHextdz = property(lambda self: self.get("dHextdz"))
    xyz = property(lambda self: self.get("positions"))

    tolerance = property(lambda self: self.get_option("tolerance"), lambda self, v: self.set_option("tolerance", v))
    max_iteration = property(lambda self: int(self.get_option("max_iteration")),
                             lambda self, v: self.set_option("max_iteration", v))
    naive = property(lambda self: bool(self.get_option("naive")), lambda self, v: self.set_option("naive", 1 if v else 0))


class mf_scene_desc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("pos", ctypes.c_void_p), ("h", ctypes.c_float), ("volume", ctypes.c_float),
                ("chi", ctypes.c_float), ("H0", ctypes.c_float * 3)]


def _batch_sigs(lib):
    i32, i64, vp, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_double
    sig = {
        "mf_batch_create": (i32, [ctypes.POINTER(mf_scene_desc), i32, i32, ctypes.POINTER(vp)]),
        "mf_batch_destroy": (i32, [vp]),
        "mf_batch_set_stream": (i32, [vp, vp]),
        "mf_batch_num_scenes": (i32, [vp, ctypes.POINTER(i32)]),
        "mf_batch_solve": (i32, [vp, i64, f64, ctypes.POINTER(i64), ctypes.POINTER(f64)]),
        "mf_batch_eval_force": (i32, [vp]),
        "mf_batch_advance": (i32, [vp, f64, i32, i32, f64, i32]),
        "mf_batch_get": (i32, [vp, i32, i32, vp]),
        "mf_batch_solver_state": (i32, [vp, vp, vp]),
        "mf_batch_get_counters": (i32, [vp, ctypes.POINTER(mf_counters)]),
        "mf_batch_reset_counters": (i32, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


class Batch:
    """Many independent scenes advanced together (mf_batch_* in mf.h)."""

    def __init__(self, scenes, device: int = 0):
        lib = load()
        _batch_sigs(lib)
        arr = (mf_scene_desc * len(scenes))()
        self._keep = []
        self.sizes = []
        for k, sc in enumerate(scenes):
            p = _f32(sc.pos)
            self._keep.append(p)
            self.sizes.append(len(p))
            arr[k].n = len(p)
            arr[k].pos = p.ctypes.data
            arr[k].h, arr[k].volume, arr[k].chi = float(sc.h), float(sc.volume), float(sc.chi)
            for j in range(3):
                arr[k].H0[j] = float(sc.H0[j])
        h = ctypes.c_void_p()
        check(lib.mf_batch_create(arr, len(scenes), int(device), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().mf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, max_iter: int = 200, rel_tol: float = 1e-6):
        it = ctypes.c_int64(0)
        worst = ctypes.c_double(0)
        st = load().mf_batch_solve(self._h, int(max_iter), float(rel_tol), ctypes.byref(it), ctypes.byref(worst))
        if st not in (MF_OK, 3):
            check(st)
        return it.value, worst.value

    def eval_force(self):
        check(load().mf_batch_eval_force(self._h))

    def advance(self, dt: float, steps: int, iters_per_step: int = 4, rel_tol: float = 1e-6, graph: bool = True):
        check(load().mf_batch_advance(self._h, float(dt), int(steps), int(iters_per_step), float(rel_tol),
                                      1 if graph else 0))

    def get(self, scene: int, quantity: str) -> np.ndarray:
        out = np.empty((self.sizes[scene], 3), dtype=np.float32)
        check(load().mf_batch_get(self._h, int(scene), Q[quantity], out.ctypes.data))
        return out

    def solver_state(self):
        n = len(self.sizes)
        rr = np.zeros(n)
        it = np.zeros(n)
        check(load().mf_batch_solver_state(self._h, rr.ctypes.data, it.ctypes.data))
        return rr, it

    def counters(self) -> dict:
        c = mf_counters()
        check(load().mf_batch_get_counters(self._h, ctypes.byref(c)))
        return {f: getattr(c, f) for f, _ in mf_counters._fields_}

    def reset_counters(self):
        check(load().mf_batch_reset_counters(self._h))


class mf_server_config(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_double), ("max_active", ctypes.c_int32),
                ("steps_per_request", ctypes.c_int32), ("iters_per_step", ctypes.c_int32), ("device", ctypes.c_int32),
                ("rel_tol", ctypes.c_double), ("dt", ctypes.c_double)]


class mf_server_stats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("running", ctypes.c_int64), ("queued", ctypes.c_int64),
                ("completed", ctypes.c_int64), ("ticks", ctypes.c_int64), ("rebatches", ctypes.c_int64),
                ("bytes_in_use", ctypes.c_double), ("field_pairs", ctypes.c_double), ("force_pairs", ctypes.c_double),
                ("busy_ms", ctypes.c_double)]


class Server:
    """Request queue with continuous batching (mf_server_* in mf.h)."""

    def __init__(self, hbm_budget_bytes=120e9, max_active=64, steps_per_request=20, iters_per_step=4,
                 rel_tol=1e-6, dt=1e-4, device=0):
        lib = load()
        i32, i64, vp, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_double
        for name, res, args in (
                ("mf_server_create", i32, [ctypes.POINTER(mf_server_config), ctypes.POINTER(vp)]),
                ("mf_server_destroy", i32, [vp]),
                ("mf_server_submit", i32, [vp, ctypes.POINTER(mf_scene_desc), ctypes.POINTER(i64)]),
                ("mf_server_step", i32, [vp, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(f64)]),
                ("mf_server_poll", i32, [vp, i64, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(f64)]),
                ("mf_server_result", i32, [vp, i64, i32, vp]),
                ("mf_server_get_stats", i32, [vp, ctypes.POINTER(mf_server_stats)]),
                ("mf_server_step_times", i32, [vp, i64, ctypes.POINTER(f64), i32, ctypes.POINTER(i32)])):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        cfg = mf_server_config(float(hbm_budget_bytes), int(max_active), int(steps_per_request), int(iters_per_step),
                               int(device), float(rel_tol), float(dt))
        h = ctypes.c_void_p()
        check(lib.mf_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.sizes = {}

    def close(self):
        if getattr(self, "_h", None):
            load().mf_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, sc) -> int:
        p = _f32(sc.pos)
        d = mf_scene_desc()
        d.n, d.pos = len(p), p.ctypes.data
        d.h, d.volume, d.chi = float(sc.h), float(sc.volume), float(sc.chi)
        for j in range(3):
            d.H0[j] = float(sc.H0[j])
        rid = ctypes.c_int64(0)
        check(load().mf_server_submit(self._h, ctypes.byref(d), ctypes.byref(rid)))
        self.sizes[rid.value] = len(p)
        return rid.value

    def step(self):
        a, c, ms = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_double(0)
        check(load().mf_server_step(self._h, ctypes.byref(a), ctypes.byref(c), ctypes.byref(ms)))
        return a.value, c.value, ms.value

    def poll(self, rid):
        st, steps, lat = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_double(0)
        check(load().mf_server_poll(self._h, int(rid), ctypes.byref(st), ctypes.byref(steps), ctypes.byref(lat)))
        return st.value, steps.value, lat.value

    def step_times(self, rid) -> np.ndarray:
        """Wall time (ms) of each timestep the request has taken so far."""
        n = ctypes.c_int32(0)
        check(load().mf_server_step_times(self._h, int(rid), None, 0, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1), dtype=np.float64)
        check(load().mf_server_step_times(self._h, int(rid), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          len(out), ctypes.byref(n)))
        return out[:n.value]

    def result(self, rid, quantity: str) -> np.ndarray:
        out = np.empty((self.sizes[rid], 3), dtype=np.float32)
        check(load().mf_server_result(self._h, int(rid), Q[quantity], out.ctypes.data))
        return out

    def stats(self) -> dict:
        s = mf_server_stats()
        check(load().mf_server_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in mf_server_stats._fields_}


class FmmMatrix:
    """FMM matrix of the field kernel over a source set and a target set: the
    replacement of fmmtl::kernel_matrix<DipoleBSpherical>(kernel, sources,
    targets) and its operator* (fmmtl/KernelMatrix.hpp:127-131).  targets=None
    means the targets are the sources."""

    def __init__(self, sources, h, targets=None, order=8, theta=0.5, leaf_min=12, device=0):
        self._h = None
        src = _f32(sources)
        tgt = None if targets is None else _f32(targets)
        self.ns = len(src)
        self.nt = self.ns if tgt is None else len(tgt)
        h_ = ctypes.c_void_p()
        check(load().mf_fmm_create(src.ctypes.data, self.ns, None if tgt is None else tgt.ctypes.data,
                                   0 if tgt is None else self.nt, float(h), int(order), float(theta), int(leaf_min),
                                   int(device), ctypes.byref(h_)))
        self._h = h_

    def field(self, charges) -> np.ndarray:
        c = _f32(charges)
        assert len(c) == self.ns
        out = np.empty((self.nt, 3), np.float32)
        check(load().mf_fmm_field(self._h, c.ctypes.data, out.ctypes.data))
        return out

    def hessian(self, charges) -> np.ndarray:
        """[nt][9] force tensors, glm column-major (entry c*3 + r)."""
        c = _f32(charges)
        assert len(c) == self.ns
        out = np.empty((self.nt, 9), np.float32)
        check(load().mf_fmm_hessian(self._h, c.ctypes.data, out.ctypes.data))
        return out

    def stats(self) -> dict:
        st = mf_fmm_stats()
        check(load().mf_fmm_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in mf_fmm_stats._fields_}

    def close(self):
        if self._h is not None:
            load().mf_fmm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_report() -> list[str]:
    """The autotuner's block-shape choices so far in this process."""
    n = ctypes.c_int64(0)
    check(load().mf_autotune_report(None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    check(load().mf_autotune_report(buf, n.value + 1, ctypes.byref(n)))
    return [ln for ln in buf.value.decode().splitlines() if ln]


def probe_fp32_peak() -> float:
    """Measured dense FP32 FMA throughput of the current device, TFLOP/s."""
    v = ctypes.c_double(0)
    check(load().mf_probe_fp32_peak(ctypes.byref(v)))
    return v.value


# -- direct evaluation on device buffers (torch CUDA tensors) -----------------
def _dev(t):
    import torch
    assert t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def direct_field(targets, sources, charges, h):
    import torch
    out = torch.empty((targets.shape[0], 3), dtype=torch.float32, device=targets.device)
    check(load().mf_direct_field(_dev(targets), targets.shape[0], _dev(sources), _dev(charges), sources.shape[0],
                                 float(h), _dev(out), _stream()))
    return out


def direct_force_tensor(targets, sources, charges, h):
    import torch
    out = torch.empty((targets.shape[0], 9), dtype=torch.float32, device=targets.device)
    check(load().mf_direct_force_tensor(_dev(targets), targets.shape[0], _dev(sources), _dev(charges),
                                        sources.shape[0], float(h), _dev(out), _stream()))
    return out


def direct_force(pos, mom, h, rext9=None, naive_quirks=False):
    import torch
    out = torch.empty((pos.shape[0], 3), dtype=torch.float32, device=pos.device)
    check(load().mf_direct_force(_dev(pos), _dev(mom), pos.shape[0], float(h),
                                 _dev(rext9) if rext9 is not None else None, 1 if naive_quirks else 0,
                                 _dev(out), _stream()))
    return out
