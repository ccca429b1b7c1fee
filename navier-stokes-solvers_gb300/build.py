"""Build recipe for libns_gb300.so (sm_103a kernels + C host drop-in).

    python navier-stokes-solvers_gb300/build.py          # build if sources changed

The CUDA translation unit is compiled with nvcc for sm_103a only; the C host
layer (reference API, forcing, config) with gcc; everything is linked into one
shared library with the CUDA runtime linked statically.  Objects go to
``_build/`` beside this file; the library beside this file.  Both are
git-ignored.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libns_gb300.so")
RUNNER = os.path.join(PKG, "ns_run")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]
CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-ffp-contract=off", "-Wall", "-I", INCLUDE]


def _sources():
    cu = sorted(glob.glob(os.path.join(PKG, "csrc", "*.cu")))
    c = sorted(glob.glob(os.path.join(PKG, "host", "*.c")))
    deps = (cu + c + glob.glob(os.path.join(PKG, "csrc", "*.cuh")) + glob.glob(os.path.join(PKG, "csrc", "*.h"))
            + glob.glob(os.path.join(PKG, "host", "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h")))
    return cu, c, deps


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_runner(force: bool = False) -> str:
    """The config-driven runner (driver/ns_run.c), linked against the library."""
    src = os.path.join(PKG, "driver", "ns_run.c")
    if force or _stale(RUNNER, [src, LIB] + glob.glob(os.path.join(INCLUDE, "*.h"))):
        _run(["gcc"] + CFLAGS + [src, "-L", PKG, "-lns_gb300", "-Wl,-rpath,$ORIGIN", "-lpthread", "-lm", "-o", RUNNER])
    return RUNNER


def build(force: bool = False, verbose: bool = False) -> str:
    cu, c, deps = _sources()
    if not force and not _stale(LIB, deps + [__file__]):
        build_runner()
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        jobs.append([NVCC] + NVFLAGS + ["-c", src, "-o", obj])
    for src in c:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        jobs.append(["gcc"] + CFLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, len(jobs))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr, file=sys.stderr)
    _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lm"])
    build_runner(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
