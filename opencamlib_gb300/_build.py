"""In-tree build of the CUDA library and the C++ facade test program.

Every translation unit is compiled for sm_103a only, in parallel, into
opencamlib_gb300/_build/.  FP64 device and host code is compiled without
multiply-add contraction (--fmad=false, -ffp-contract=off) so the contact
arithmetic rounds like the reference; FP32 screening code asks for fused
multiply-adds explicitly where it wants them.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libocl_gb300.so")
FACADE_TEST = os.path.join(OUT, "facade_test")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(ROOT, "include", "ocl_gb300.h")]
    objs = []
    jobs = []
    for s in sources:
        o = os.path.join(OUT, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", s, "-o", o] + (["-Xptxas", "-v"] if verbose else []))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
        if verbose:
            for lg in logs:
                print(lg)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


def build_facade_test() -> str | None:
    """Compile tests/facade_test.cpp against the C++ facade headers and link
    it to the library (host compiler only)."""
    src = os.path.join(ROOT, "tests", "facade", "facade_test.cpp")
    if not os.path.exists(src):
        return None
    inc = os.path.join(PKG, "include")
    deps = [src] + glob.glob(os.path.join(inc, "ocl", "*.hpp")) + [LIB]
    if _stale(FACADE_TEST, deps):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", inc, "-I", os.path.join(ROOT, "include"), src,
              "-o", FACADE_TEST, "-L", OUT, "-locl_gb300", f"-Wl,-rpath,{OUT}"])
    return FACADE_TEST
