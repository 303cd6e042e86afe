"""Build the CUDA library in-tree: robust-implicit-surface-networks_gb300/_build/libria.so, plus the
C++ host layer over its C ABI (_build/libria_host.so) and the two command-line programs
(_build/impl_arrangement, _build/material_interface).

sm_103a only (GB300).  The translation units compile in parallel; every kernel is built with
-fmad=false so that each FP64 operation is rounded on its own (the sampled values and vertex
coordinates must round exactly as the reference formulas written out in C++ do); fused
multiply-adds appear only where the code calls fma() explicitly (exact products).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libria.so")
SOURCES = ["k_ab.cu", "k_cut.cu", "k_extract.cu", "k_extract_mi.cu", "k_noalloc.cu", "k_tetmaps.cu", "k_connect.cu", "capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-fmad=false", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]
HOST = os.path.join(HERE, "host")
HOST_LIB = os.path.join(OUT_DIR, "libria_host.so")
HOST_SOURCES = ["ria_host.cpp", "mesh_io.cpp"]
APPS = ["impl_arrangement", "material_interface", "csg"]
CXX = os.environ.get("CXX", "g++")
# -ffp-contract=off: the grid coordinates and unit axis vectors round as written (aarch64 g++
# contracts a*b+c into fma by default)
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "ria.h"))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _host_stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".hpp")]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "ria.h"))
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(jobs, what, verbose):
    if not jobs:
        return
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for cmd, r in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if r.returncode != 0:
                raise RuntimeError("%s failed: %s\n%s%s" % (what, " ".join(cmd), r.stdout, r.stderr))
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s.replace(".cu", ".o"))
        if _stale(obj, src):
            jobs.append([cc, *ARCH, *FLAGS, "-c", src, "-o", obj])
    host_objs = []
    for s in HOST_SOURCES:
        src = os.path.join(HOST, s)
        obj = os.path.join(OUT_DIR, s.replace(".cpp", ".o"))
        host_objs.append(obj)
        if _host_stale(obj, [src]):
            jobs.append([CXX, *HOST_FLAGS, "-c", src, "-o", obj])
    _run(jobs, "compile", verbose)
    objs = [os.path.join(OUT_DIR, s.replace(".cu", ".o")) for s in SOURCES]
    relinked = False
    if any(j[0] == cc for j in jobs) or not os.path.exists(LIB):
        _run([[cc, *ARCH, "-shared", *objs, "-ldl", "-o", LIB]], "link", verbose)  # -ldl: NVTX loads its tool
        relinked = True
    if relinked or _host_stale(HOST_LIB, host_objs):
        _run([[CXX, "-shared", "-pthread", *host_objs, "-L" + OUT_DIR, "-lria", "-Wl,-rpath,$ORIGIN", "-o", HOST_LIB]],
             "link", verbose)
        relinked = True
    apps = []
    for app in APPS:
        src = os.path.join(HOST, "apps", app + ".cpp")
        exe = os.path.join(OUT_DIR, app)
        if relinked or _host_stale(exe, [src]):
            apps.append([CXX, *HOST_FLAGS, src, "-L" + OUT_DIR, "-lria_host", "-lria", "-Wl,-rpath,$ORIGIN", "-o", exe])
    _run(apps, "build", verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
