"""ctypes wrapper of ref_harness.cpp: the reference's own CUDA kernels (cubins compiled from the
reference sources by build_ref.sh) driven on the same host arrays as the product.

TEST INFRASTRUCTURE ONLY (the GPU-side oracle for the 1e-12 / identical-switch parity gate).
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", platform.machine(), "libref_harness.so")
REF_DIR = os.path.join(HERE, "_ref")
_lib = None


def cubin_path():
    for tag in ("sm_100", "sm_103a"):
        p = os.path.join(REF_DIR, f"ref_{tag}.cubin")
        if os.path.exists(p):
            return p
    return None


def available():
    return cubin_path() is not None and os.path.exists(LIB_PATH)


def build():
    """Compile the harness host code (needs the CUDA toolkit headers and libcuda)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    src = os.path.join(HERE, "ref_harness.cpp")
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", f"-I{cuda}/include", src, "-o", LIB_PATH,
           f"-L{cuda}/lib64/stubs", f"-L{cuda}/lib64", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

        L = C.CDLL(LIB_PATH)
        L.refh_last_error.restype = C.c_char_p
        L.refh_create.argtypes = [C.c_char_p, C.POINTER(_ffi.FieldPointer), C.POINTER(_ffi.FieldSizes),
                                  C.POINTER(C.c_void_p)]
        L.refh_stage.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                 C.POINTER(_ffi.FieldPointer)]
        L.refh_evolve.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_float)]
        L.refh_adjust_dt.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]
        L.refh_download.argtypes = [C.c_void_p, C.POINTER(_ffi.FieldPointer)]
        L.refh_upload_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.refh_destroy.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _ck(rc):
    if rc != 0:
        raise RuntimeError("reference harness: " + lib().refh_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data


class RefKernels:
    """The reference solver's device side (GPUevolve.cu) on one case."""

    def __init__(self, hf, cubin=None):
        from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

        self.hf = hf
        self._fp = hf.to_c()
        sz = _ffi.FieldSizes(*[hf.sizes[n] for n, _ in _ffi.FieldSizes._fields_])
        self._sz = sz
        self.h = C.c_void_p()
        _ck(lib().refh_create((cubin or cubin_path()).encode(), C.byref(self._fp), C.byref(sz), C.byref(self.h)))

    def stage(self, k, R, Cv, dt, store=None):
        from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

        names = ["faceFD", "gradFD", "limiter", "shockIndicator", "Flux", "Res", "FD", "cFD"]
        out = self.hf.empty_like_outputs(names)
        fp = _ffi.FieldPointer()
        for n in names:
            setattr(fp, n, _p(out[n]))
        _ck(lib().refh_stage(self.h, k, R, Cv, dt, int(k == 2 if store is None else store), C.byref(fp)))
        return out

    def evolve(self, nsteps, R, Cv, dt):
        ms = C.c_float()
        _ck(lib().refh_evolve(self.h, nsteps, R, Cv, dt, C.byref(ms)))
        return ms.value

    def adjust_dt(self, R, Cv, CFL):
        d = C.c_double()
        _ck(lib().refh_adjust_dt(self.h, R, Cv, CFL, C.byref(d)))
        return d.value

    def state(self):
        from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

        out = self.hf.empty_like_outputs(["FD", "cFD", "shockIndicator", "matrix"])
        fp = _ffi.FieldPointer()
        for n in out:
            setattr(fp, n, _p(out[n]))
        _ck(lib().refh_download(self.h, C.byref(fp)))
        return out

    def upload_state(self, FD=None, cFD=None, cFDold=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (FD, cFD, cFDold)]
        _ck(lib().refh_upload_state(self.h, *[_p(a) for a in arrs]))

    def close(self):
        if self.h:
            lib().refh_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
