"""Builds libmce_gb300.so in-tree (cauchyfriendly_gb300/_build) for sm_103a.

The kernels are compiled with --fmad=false and the host side with
-ffp-contract=off: the estimator's integer structure (coalignment, term
reduction, vertex selection) is decided by floating-point comparisons, and
unfused multiply-add keeps those decisions identical to the reference's
double-precision C++ on every host.

The kernel translation units are split by state dimension so they compile in
parallel (a minute or two on either host).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmce_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
DIMS = list(range(1, 9))


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I" + CSRC, "-I" + os.path.join(os.path.dirname(HERE), "include")]


def _sources():
    srcs = [os.path.join(CSRC, f) for f in ("mce_kernels.cu", "mce_engine.cu", "mce_no_alloc.cu", "mce_host.cpp",
                                            "mce_adjoint.cu", "mce_ndpdf.cu")]
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(os.path.dirname(HERE), "include", "mce_c_api.h"))
    return srcs, hdrs


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    srcs, hdrs = _sources()
    return any(os.path.getmtime(f) > t for f in srcs + hdrs + [__file__])


def build(force=False, verbose=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    # kernels: one object per state dimension so the instantiations compile in parallel
    for d in DIMS:
        obj = os.path.join(OUT, "mce_kernels_d%d.o" % d)
        objs.append(obj)
        jobs.append([nvcc, "-c", os.path.join(CSRC, "mce_kernels.cu"), "-o", obj, "-DMCE_ONLY_DIM=%d" % d]
                    + _flags())
    obj = os.path.join(OUT, "mce_kernels_common.o")
    objs.append(obj)
    jobs.append([nvcc, "-c", os.path.join(CSRC, "mce_kernels.cu"), "-o", obj, "-DMCE_ONLY_DIM=0"] + _flags())
    for d in DIMS:
        obj = os.path.join(OUT, "mce_engine_d%d.o" % d)
        objs.append(obj)
        jobs.append([nvcc, "-c", os.path.join(CSRC, "mce_engine.cu"), "-o", obj, "-DMCE_ONLY_DIM=%d" % d]
                    + _flags())
    obj = os.path.join(OUT, "mce_engine_common.o")
    objs.append(obj)
    jobs.append([nvcc, "-c", os.path.join(CSRC, "mce_engine.cu"), "-o", obj, "-DMCE_ONLY_DIM=0"] + _flags())
    obj = os.path.join(OUT, "mce_no_alloc.o")
    objs.append(obj)
    jobs.append([nvcc, "-c", os.path.join(CSRC, "mce_no_alloc.cu"), "-o", obj] + _flags())
    obj = os.path.join(OUT, "mce_ndpdf.o")
    objs.append(obj)
    jobs.append([nvcc, "-c", os.path.join(CSRC, "mce_ndpdf.cu"), "-o", obj] + _flags())
    obj = os.path.join(OUT, "mce_adjoint.o")
    objs.append(obj)
    jobs.append([nvcc, "-c", os.path.join(CSRC, "mce_adjoint.cu"), "-o", obj] + _flags())
    # host-only C++ (window managers, Speyer restart)
    obj = os.path.join(OUT, "mce_host.o")
    objs.append(obj)
    jobs.append([nvcc, "-c", os.path.join(CSRC, "mce_host.cpp"), "-o", obj] + _flags())
    ncpu = max(1, os.cpu_count() or 1)
    running = []
    pending = list(jobs)
    failed = None
    while pending or running:
        while pending and len(running) < ncpu:
            j = pending.pop(0)
            if verbose:
                print(" ".join(j))
            running.append((j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        j, p = running.pop(0)
        out, _ = p.communicate()
        if p.returncode != 0 and failed is None:
            failed = (j, out.decode())
        elif verbose and out:
            print(out.decode())
    if failed:
        raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(failed[0]), failed[1]))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stdout.decode()))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
