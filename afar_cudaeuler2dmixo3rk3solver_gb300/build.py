"""Build recipe for libafar (the product) and the oracle (test infrastructure).

nvcc compiles the CUDA translation units for sm_103a only; g++ compiles the host precompute with
OpenMP and -ffp-contract=off (identical arrays on x86 and aarch64 hosts).  Objects go to
``_build/<machine>/`` in the package; the shared library lands beside them (per host architecture) and is
loaded in-tree.  Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build", platform.machine())
LIB = os.path.join(BUILD, "libafar.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", platform.machine(), "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_lib(force=False, verbose=False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "afar.h"))
    units = [
        ("afar_solver.cu", "nvcc"),
        ("afar_noalloc.cu", "nvcc"),
        ("afar_peak.cu", "nvcc"),
        ("afar_precompute_gpu.cu", "nvcc_nofma"),
        ("afar_precompute.cpp", "cxx"),
        ("afar_error.cpp", "cxx"),
        ("afar_server.cpp", "cxx"),
    ]
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src, kind in units:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            if kind == "nvcc":
                cmd = [nvcc] + NVCC_FLAGS + ["-c", s, "-o", o]
            elif kind == "nvcc_nofma":  # bit-identical to the host precompute (-ffp-contract=off)
                cmd = [nvcc] + NVCC_FLAGS + ["-fmad=false", "-c", s, "-o", o]
            else:
                cmd = ["g++"] + CXX_FLAGS + ["-c", s, "-o", o]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", LIB] + objs + ["-lgomp", "-lpthread"])
    return LIB


def build_oracle(force=False) -> str:
    srcs = [os.path.join(ORACLE_DIR, f) for f in ("afar_oracle.c", "afar_oracle_stage.inc", "afar_oracle.h")]
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    if force or _stale(ORACLE_LIB, srcs + [os.path.join(ROOT, "include", "afar.h")]):
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
              os.path.join(ORACLE_DIR, "afar_oracle.c"), "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def build_all(force=False, verbose=False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_lib, force, verbose)
        f2 = ex.submit(build_oracle, force)
        return f1.result(), f2.result()


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv, verbose="-v" in sys.argv))
