"""Build libmfgb.so (the sm_103a CUDA library behind include/mf.h) in-tree.

Every .cu under csrc/ is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked with the static
CUDA runtime into ``libmfgb.so`` next to this file.  Objects go to ``_build/``.
Rebuilds only what changed (source or header newer than the object).  A
stamp in ``_build/`` records the machine, the nvcc version and the flags that
built the objects; when any of them differs (objects carried from another
host, a new toolkit) everything is rebuilt.  Objects whose source is gone are
deleted, so they cannot be linked in.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmfgb.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(src: str, obj: str, hdr_mtime: float) -> bool:
    if not os.path.exists(obj):
        return True
    m = os.path.getmtime(obj)
    return os.path.getmtime(src) > m or hdr_mtime > m


def _compile(src: str, obj: str, extra: list[str]) -> None:
    cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")


def _toolchain_stamp(extra: list[str]) -> str:
    r = subprocess.run([nvcc(), "--version"], capture_output=True, text=True)
    text = "\n".join([platform.machine(), r.stdout.strip(), " ".join(NVCC_FLAGS + extra)])
    return hashlib.sha256(text.encode()).hexdigest()


def build(verbose: bool = False, extra: list[str] | None = None, force: bool = False) -> str:
    extra = extra or []
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    names = {os.path.basename(s)[:-3] + ".o" for s in srcs}
    for o in glob.glob(os.path.join(BUILD, "*.o")):
        if os.path.basename(o) not in names:
            os.remove(o)
    stamp_path = os.path.join(BUILD, "toolchain.stamp")
    stamp = _toolchain_stamp(extra)
    old = open(stamp_path).read().strip() if os.path.exists(stamp_path) else ""
    if old != stamp:
        force = True
    hdr = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(s, o, hdr):
            jobs.append((s, o))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            futs = [ex.submit(_compile, s, o, extra) for s, o in jobs]
            for f in futs:
                f.result()
    newest = max(os.path.getmtime(o) for o in objs)
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if old != stamp:
        with open(stamp_path, "w") as f:
            f.write(stamp + "\n")
    if verbose:
        print(f"built {LIB} ({len(jobs)} objects recompiled)")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
