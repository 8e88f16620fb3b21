"""vtg_build.py -- builds libvtg.so in place: every CUDA source under csrc/ for sm_103a, compiled in parallel with nvcc,
then linked into one shared library beside this file. Rebuilds only what changed.

    python vtg_build.py            # or: import vtg_build; vtg_build.build()
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvtg.so")
CHECKED_LIB = os.path.join(HERE, "libvtg_checked.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: the kernels write every fused multiply-add they mean; nothing else is contracted.
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-I" + INCLUDE,
           "--expt-relaxed-constexpr"]
CFLAGS = ["-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wextra", "-I" + INCLUDE, "-ffp-contract=off"]


def _nvcc() -> str:
    for p in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + \
        glob.glob(os.path.join(HOST, "*.h"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + _headers())


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(verbose: bool = False, extra=(), checked: bool = False) -> str:
    """libvtg.so; with checked=True the separate libvtg_checked.so, whose LK patch operations test every window they
    read against the level's bounds and record a failure instead of reading (-DVTG_CHECKED)."""
    obj_dir = OBJ + "_checked" if checked else OBJ
    lib = CHECKED_LIB if checked else LIB
    extra = tuple(extra) + (("-DVTG_CHECKED",) if checked else ())
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = _nvcc()
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(obj_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append([nvcc, *ARCH, *NVFLAGS, *extra, "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(HOST, "*.c"))):
        obj = os.path.join(obj_dir, os.path.basename(src)[:-2] + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append(["cc", *CFLAGS, "-I" + "/usr/local/cuda/include", "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for log in ex.map(_compile, jobs):
            if verbose and log:
                print(log, file=sys.stderr)
    if jobs or not os.path.exists(lib):
        cmd = [nvcc, *ARCH, "-shared", "-o", lib, *objs, "-lcudart", "-lpthread"]
        _compile(cmd)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, extra=tuple(sys.argv[1:])))
