"""ctypes wrapper of the CPU oracle (oracle/afar_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, as the checker and the timed CPU restatement.  The product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import platform

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", platform.machine(), "liboracle.so")
_p = C.c_void_p


class OracleMesh(C.Structure):
    _fields_ = [("Nc", C.c_int), ("Nf", C.c_int), ("Nb", C.c_int), ("maxS", C.c_int), ("maxM", C.c_int)] + [
        (n, _p) for n in ("CELL", "FACE", "V", "neighbour", "bnei", "btype", "S", "M", "cellFaces", "gsten", "rbf32",
                          "rbf64", "mat32", "mat64")]


class OracleWork(C.Structure):
    _fields_ = [(n, _p) for n in ("grad", "lim", "faceFD", "Flux", "Res")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        L.oracle_resolve_stencil.argtypes = [C.c_int, C.c_int, C.c_int, _p, _p, _p, _p]
        L.oracle_ls_matrix.argtypes = [C.POINTER(OracleMesh), _p, _p]
        for pol in ("ref", "fp64"):
            getattr(L, f"oracle_reconstruct_{pol}").argtypes = [C.POINTER(OracleMesh), _p, _p, _p, _p, _p]
            getattr(L, f"oracle_bvd_{pol}").argtypes = [C.POINTER(OracleMesh), _p, _p, _p, _p, _p]
            getattr(L, f"oracle_flux_{pol}").argtypes = [C.POINTER(OracleMesh), _p, _p, _p, _p, _p, C.c_double,
                                                         C.c_double, _p]
            getattr(L, f"oracle_evolve_{pol}").argtypes = [C.POINTER(OracleMesh), _p, _p, _p, _p,
                                                           C.POINTER(OracleWork), C.c_double, C.c_double, C.c_double,
                                                           C.c_int]
        L.oracle_reconstruct_gauss_fp64.argtypes = [C.POINTER(OracleMesh), _p, _p, C.c_int, _p, _p, _p]
        L.oracle_flux_gauss_fp64.argtypes = [C.POINTER(OracleMesh), _p, _p, _p, _p, _p, C.c_int, _p, _p, C.c_double,
                                             C.c_double, _p]
        L.oracle_evolve_gauss_fp64.argtypes = [C.POINTER(OracleMesh), _p, _p, _p, _p, C.POINTER(OracleWork),
                                               C.c_double, C.c_double, C.c_double, C.c_int, _p, _p, _p, _p]
        L.oracle_residual.argtypes = [C.POINTER(OracleMesh), _p, _p]
        L.oracle_update.argtypes = [C.POINTER(OracleMesh), _p, _p, _p, _p] + [C.c_double] * 6
        L.oracle_boundary.argtypes = [C.POINTER(OracleMesh), _p, C.c_double, C.c_double]
        L.oracle_delta_t.argtypes = [C.POINTER(OracleMesh), _p, C.c_double, C.c_double, C.c_double]
        L.oracle_delta_t.restype = C.c_double
        L.oracle_max_threads.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class Oracle:
    """The oracle bound to one case (the reference's host arrays in a HostFields)."""

    BETA = ((1.0, 0.0, 1.0), (0.75, 0.25, 0.25), (0.333333, 0.666667, 0.666667))

    def __init__(self, hf, R, Cv, policy="ref", matrix32=None, gauss_flux=False):
        """gauss_flux: the library's optional multi-point face flux (fp64 policy only), with the
        bundle's faceGaussPoints / faceGaussWeights / RBFbasisGauss64."""
        s = hf.sizes
        self.gauss = None
        if gauss_flux:
            if policy != "fp64":
                raise ValueError("the multi-point face flux oracle is FP64")
            pts = np.ascontiguousarray(hf.a["faceGaussPoints"], dtype=np.float64)
            w = np.asarray(hf.a["faceGaussWeights"][0], dtype=np.float64) if hf.a["faceGaussWeights"].size else \
                np.ones(pts.shape[1])
            self.gauss = (pts.shape[1], np.ascontiguousarray(hf.a["RBFbasisGauss64"]), pts,
                          np.ascontiguousarray(w / w.sum()))
        self.hf = hf
        self.R, self.Cv = float(R), float(Cv)
        self.policy = policy
        self.Nc, self.Nf, self.Nb = s["cellsNum"], s["facesNum"], s["totalBoundaryFacesNum"]
        self.maxS, self.maxM = s["maxStencilSize"], s["maxCompactStencilSize"]
        self.gsten = np.zeros(self.maxS * self.Nc, dtype=np.int32)
        lib().oracle_resolve_stencil(self.Nc, self.maxS, s["maxLocalBlockStencilSize"], _ptr(hf.stencilSize),
                                     _ptr(hf.localStencil), _ptr(hf.extendStencil), _ptr(self.gsten))
        self.mat64 = np.zeros(2 * self.maxM * self.Nc)
        self.mat32 = np.zeros(2 * self.maxM * self.Nc, dtype=np.float32)
        self._keep = []
        m = self._mesh()
        lib().oracle_ls_matrix(C.byref(m), _ptr(self.mat64), _ptr(self.mat32))
        if matrix32 is not None:  # run on the matrix some other builder produced
            self.mat32 = np.ascontiguousarray(matrix32, dtype=np.float32)
        self.rbf64 = hf.a.get("RBFbasis64")
        if self.rbf64 is None:
            self.rbf64 = hf.RBFbasis.astype(np.float64)
        self.m = self._mesh()

    def _mesh(self):
        hf = self.hf
        m = OracleMesh()
        m.Nc, m.Nf, m.Nb, m.maxS, m.maxM = self.Nc, self.Nf, self.Nb, self.maxS, self.maxM
        m.CELL, m.FACE, m.V = _ptr(hf.CELL), _ptr(hf.FACE), _ptr(hf.cellVolume)
        m.neighbour, m.bnei, m.btype = _ptr(hf.neighbour), _ptr(hf.boundaryFaceNeiLabel), _ptr(hf.boundaryFacesType)
        m.S, m.M, m.cellFaces, m.gsten = _ptr(hf.stencilSize), _ptr(hf.compactStencilSize), _ptr(hf.cellFaces), _ptr(
            self.gsten)
        m.rbf32 = _ptr(hf.RBFbasis)
        rb = getattr(self, "rbf64", None)
        m.rbf64 = _ptr(rb if rb is not None else hf.RBFbasis.astype(np.float64))
        m.mat32, m.mat64 = _ptr(self.mat32), _ptr(self.mat64)
        if rb is None:
            self._keep.append(hf.RBFbasis.astype(np.float64))
            m.rbf64 = _ptr(self._keep[-1])
        return m

    def lim_dtype(self):
        return np.float32 if self.policy == "ref" else np.float64

    def new_state(self):
        hf = self.hf
        return {"FD": hf.FD.copy(), "cFD": hf.cFD.copy(), "cFDold": hf.cFD.copy(),
                "si": np.zeros(2 * (self.Nc + self.Nb), dtype=np.int8)}

    def stage(self, st, k, dt):
        """One RK stage with every intermediate returned (the parity-test view)."""
        pol = self.policy
        L = lib()
        grad = np.zeros((self.Nc, 8))
        lim = np.zeros((self.Nc, 4), dtype=self.lim_dtype())
        fv = np.zeros((2 * self.Nf, 4))
        flux = np.zeros((self.Nf + self.Nb, 4))
        res = np.zeros((self.Nc, 4))
        FD, cFD, cFDold, si = st["FD"], st["cFD"], st["cFDold"], st["si"]
        getattr(L, f"oracle_reconstruct_{pol}")(C.byref(self.m), _ptr(FD), _ptr(grad), _ptr(lim), _ptr(fv), _ptr(si))
        raw_lim = lim.copy()
        if self.gauss:
            ng, rbfg, gpts, gw = self.gauss
            fvg = np.zeros((2 * self.Nf, ng, 4))
            L.oracle_reconstruct_gauss_fp64(C.byref(self.m), _ptr(FD), _ptr(grad), ng, _ptr(rbfg), _ptr(gpts),
                                            _ptr(fvg))
        getattr(L, f"oracle_bvd_{pol}")(C.byref(self.m), _ptr(FD), _ptr(grad), _ptr(lim), _ptr(fv), _ptr(si))
        if self.gauss:
            L.oracle_flux_gauss_fp64(C.byref(self.m), _ptr(FD), _ptr(grad), _ptr(lim), _ptr(fvg), _ptr(si), ng,
                                     _ptr(gpts), _ptr(gw), self.R, self.Cv, _ptr(flux))
        else:
            getattr(L, f"oracle_flux_{pol}")(C.byref(self.m), _ptr(FD), _ptr(grad), _ptr(lim), _ptr(fv), _ptr(si),
                                             self.R, self.Cv, _ptr(flux))
        L.oracle_residual(C.byref(self.m), _ptr(flux), _ptr(res))
        res_out = res.copy()
        b1, b2, b3 = self.BETA[k]
        gamma = self.R / self.Cv + 1.0
        L.oracle_update(C.byref(self.m), _ptr(FD), _ptr(cFD), _ptr(cFDold), _ptr(res), self.R, gamma, dt, b1, b2, b3)
        L.oracle_boundary(C.byref(self.m), _ptr(FD), self.R, self.Cv)
        if k == 2:
            cFDold[:] = cFD
        return {"gradFD": grad, "limiter_raw": raw_lim, "limiter": lim, "faceFD": fv, "Flux": flux, "Res": res_out,
                "shockIndicator": si.copy(), "FD": FD.copy(), "cFD": cFD.copy()}

    def delta_t(self, FD, cfl):
        return lib().oracle_delta_t(C.byref(self.m), _ptr(FD), self.R, self.Cv, cfl)

    def evolve(self, st, dt, exact_rk=False):
        work = OracleWork()
        bufs = [np.zeros((self.Nc, 8)), np.zeros((self.Nc, 4), dtype=self.lim_dtype()), np.zeros((2 * self.Nf, 4)),
                np.zeros((self.Nf + self.Nb, 4)), np.zeros((self.Nc, 4))]
        work.grad, work.lim, work.faceFD, work.Flux, work.Res = [_ptr(b) for b in bufs]
        if self.gauss:
            ng, rbfg, gpts, gw = self.gauss
            fvg = np.zeros((2 * self.Nf, ng, 4))
            lib().oracle_evolve_gauss_fp64(C.byref(self.m), _ptr(st["FD"]), _ptr(st["cFD"]), _ptr(st["cFDold"]),
                                           _ptr(st["si"]), C.byref(work), self.R, self.Cv, dt, ng, _ptr(rbfg),
                                           _ptr(gpts), _ptr(gw), _ptr(fvg))
            return
        getattr(lib(), f"oracle_evolve_{self.policy}")(C.byref(self.m), _ptr(st["FD"]), _ptr(st["cFD"]),
                                                      _ptr(st["cFDold"]), _ptr(st["si"]), C.byref(work), self.R,
                                                      self.Cv, dt, int(exact_rk))


def set_threads(n):
    lib().oracle_set_threads(int(n))


def max_threads():
    return lib().oracle_max_threads()
