"""In-tree build of libmrgpu.so for sm_103a (nvcc, no cmake).

Translation units are compiled in parallel; only changed sources are rebuilt.
The library lands in ``multiregionfoam_gb300/_lib/libmrgpu.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libmrgpu.so")

SOURCES = ["kernels.cu", "engine.cu", "api.cu", "noalloc.cu", "dn.cu", "ggi_build.cu", "mono.cu", "gamg.cu", "blockpc.cu", "plan.cpp", "server.cpp", "block.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is compiled without floating-point contraction, so host arithmetic
# (GAMG's face weights) rounds the same on x86-64 and aarch64
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", CSRC, "-I", INCLUDE]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmrgpu")


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + hdrs):
            cmd = [cc] + ARCH + COMMON + ["-c", path, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [cc] + COMMON + ["-x", "c++", "-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"])
    build_adapter(force)
    return LIB


FOAM = os.path.join(HERE, "foam")
ADAPTER = os.path.join(OUT, "test_adapter")


def build_adapter(force: bool = False) -> str:
    """The lduMatrix::solver adapters + their driver, against the API shim."""
    srcs = [os.path.join(FOAM, "gpuLduSolvers.C"), os.path.join(FOAM, "test_adapter.C")]
    deps = srcs + [os.path.join(FOAM, "shim", "lduMatrix.H"), os.path.join(INCLUDE, "mrgpu.h"), LIB]
    if force or _stale(ADAPTER, deps):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(FOAM, "shim"), "-I", INCLUDE] + srcs + \
              ["-L", OUT, "-lmrgpu", "-Wl,-rpath," + OUT, "-o", ADAPTER]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("adapter build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return ADAPTER
