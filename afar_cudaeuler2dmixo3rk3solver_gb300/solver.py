"""Host-side mirror of the reference's solver object over the libafar C ABI.

``HostFields`` is the reference's host ``fieldPointer`` as numpy arrays (basicDataStructure.h).
``precompute`` does what ``basicCUDAsolver::initFieldInfo`` + ``initStencilData`` do with OpenFOAM
(basicCUDAsolver.cpp:122-851), in native code.  ``CudaSolver`` follows ``basicCUDAsolver``
(basicCUDAsolver.h:44-52): construct = precompute + both ``setDeviceFieldData`` uploads,
``set_delta_t`` = ``adjustTimeStep``, ``evolve(dt)`` = ``GPUevolve``, ``write_field`` =
``copyFieldDataDeviceToHost``; plus ``run`` (graph-captured multi-step with a device-side CFL
step) and ``stage_debug`` (per-stage intermediates for parity checks).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import hashlib
import os

import numpy as np

from . import _ffi
from ._ffi import check, lib, ptr
from .mesh import FoamMesh

_MEMBERS = [f[0] for f in _ffi.FieldPointer._fields_]


@dataclasses.dataclass
class CaseConfig:
    """fvSchemes/controlDict settings the reference reads (basicCUDAsolver.cpp:55-68)."""
    R: float = 1.0 / 1.4
    Cv: float = 1.0 / 1.4 / 0.4
    CFL: float = 0.5
    shapeFactor: float = 10.0
    stencilType: str = "edgeNeighbour"
    cOrder: int = 5
    fOrder: int = 4
    nThreads: int = 0

    def to_c(self):
        c = _ffi.CaseConfig()
        c.R, c.Cv, c.CFL, c.shapeFactor = self.R, self.Cv, self.CFL, self.shapeFactor
        c.stencilType = {"faceNeighbour": 0, "edgeNeighbour": 1}[self.stencilType]
        c.cOrder, c.fOrder, c.nThreads = self.cOrder, self.fOrder, self.nThreads
        return c


SIZE_KEYS = ["cellsNum", "facesNum", "patchesNum", "totalBoundaryFacesNum", "maxStencilSize",
             "maxCompactStencilSize", "maxLocalBlockStencilSize", "maxCompactLocalBlockStencilSize"]


class HostFields:
    """The reference's host field bundle as numpy arrays plus its integer sizes."""

    def __init__(self, sizes: dict, arrays: dict, period=(0.0, 0.0)):
        self.sizes = dict(sizes)
        self.a = dict(arrays)
        self.period = tuple(float(v) for v in period)  # of a periodic mesh

    def __getattr__(self, k):
        a = self.__dict__.get("a", {})
        if k in a:
            return a[k]
        raise AttributeError(k)

    @property
    def nc(self):
        return self.sizes["cellsNum"]

    def save(self, path: str):
        """The whole bundle (operators, RBF weights, initial fields) in one .npz file."""
        np.savez(path, __sizes__=np.array([self.sizes[k] for k in SIZE_KEYS], dtype=np.int64),
                 __period__=np.array(self.period, dtype=np.float64),
                 **{f"a_{k}": v for k, v in self.a.items()})

    @classmethod
    def load(cls, path: str) -> "HostFields":
        z = np.load(path)
        sizes = dict(zip(SIZE_KEYS, (int(v) for v in z["__sizes__"])))
        period = tuple(z["__period__"]) if "__period__" in z.files else (0.0, 0.0)
        return cls(sizes, {k[2:]: np.ascontiguousarray(z[k]) for k in z.files if k.startswith("a_")}, period)

    @property
    def nf(self):
        return self.sizes["facesNum"]

    @property
    def nb(self):
        return self.sizes["totalBoundaryFacesNum"]

    def shapes(self):
        s = self.sizes
        nc, nf, nb = s["cellsNum"], s["facesNum"], s["totalBoundaryFacesNum"]
        maxS, maxM, maxLB = s["maxStencilSize"], s["maxCompactStencilSize"], s["maxLocalBlockStencilSize"]
        nblk = (nc + _ffi.BLOCKDIM - 1) // _ffi.BLOCKDIM
        return {
            "CELL": ((nc + nb, 2), np.float64), "FACE": ((nf + nb, 5), np.float64), "cellVolume": ((nc,), np.float64),
            "FD": ((nc + nb, 4), np.float64), "limiter": ((nc, 4), np.float32),
            "shockIndicator": ((2 * (nc + nb),), np.int8), "cFD": ((nc, 4), np.float64),
            "cFDold": ((nc, 4), np.float64), "gradFD": ((nc, 8), np.float64), "Flux": ((nf + nb, 4), np.float64),
            "Res": ((nc, 4), np.float64), "neighbour": ((2 * nf,), np.int32),
            "boundaryFacesNum": ((s["patchesNum"],), np.int32), "boundaryFaceNeiLabel": ((nb,), np.int32),
            "boundaryFacesType": ((nb,), np.uint8), "stencilSize": ((nc,), np.uint8),
            "compactStencilSize": ((nc,), np.uint8), "RBFbasis": ((2 * (maxS + 1) * nf,), np.float32),
            "faceFD": ((2 * nf, 4), np.float64), "extendStencil": (((maxLB - _ffi.BLOCKDIM) * nblk,), np.int32),
            "extendStencilSize": ((nblk,), np.uint16), "compactExtendStencilSize": ((nblk,), np.uint16),
            "localStencil": ((maxS * nc,), np.uint16), "matrix": ((2 * maxM * nc,), np.float32),
            "cellFaces": ((maxM * nc,), np.int32), "minDeltaT": (((nf + 1023) // 1024,), np.float64),
        }

    def empty_like_outputs(self, names):
        sh = self.shapes()
        return {n: np.zeros(sh[n][0], dtype=sh[n][1]) for n in names}

    def to_c(self, only=None):
        fp = _ffi.FieldPointer()
        for n in _MEMBERS:
            if only is not None and n not in only:
                continue
            a = self.a.get(n)
            if a is not None:
                setattr(fp, n, ptr(np.ascontiguousarray(a)) if a.flags["C_CONTIGUOUS"] else None)
        return fp

    @staticmethod
    def from_c(fp: _ffi.FieldPointer, sz: _ffi.FieldSizes):
        sizes = {n: getattr(sz, n) for n, _ in _ffi.FieldSizes._fields_}
        hf = HostFields(sizes, {})
        for n, (shape, dt) in hf.shapes().items():
            p = getattr(fp, n)
            count = int(np.prod(shape))
            if p is None or count == 0:
                hf.a[n] = np.zeros(shape, dtype=dt)
                continue
            buf = (C.c_byte * (count * np.dtype(dt).itemsize)).from_address(p)
            hf.a[n] = np.frombuffer(buf, dtype=dt).reshape(shape).copy()
        return hf


def poly_mesh_c(mesh: FoamMesh):
    """afar_polyMesh view of a FoamMesh; returns (struct, keep-alive list)."""
    keep = [np.ascontiguousarray(mesh.points, dtype=np.float64), np.ascontiguousarray(mesh.cell_ptr, dtype=np.int32),
            np.ascontiguousarray(mesh.cell_pts, dtype=np.int32), np.ascontiguousarray(mesh.face_pts, dtype=np.int32),
            np.ascontiguousarray(mesh.owner, dtype=np.int32), np.ascontiguousarray(mesh.neighbour, dtype=np.int32),
            np.array([p[2] for p in mesh.patches], dtype=np.int32),
            np.array([p[3] for p in mesh.patches], dtype=np.int32),
            np.array([p[1] for p in mesh.patches], dtype=np.int32)]
    m = _ffi.PolyMesh()
    m.nPoints = keep[0].shape[0]
    m.points = ptr(keep[0])
    m.nCells = keep[1].shape[0] - 1
    m.cellPointsOffset = ptr(keep[1])
    m.cellPoints = ptr(keep[2])
    m.nInternalFaces = keep[5].shape[0]
    m.nFaces = keep[4].shape[0]
    m.facePoints = ptr(keep[3])
    m.owner = ptr(keep[4])
    m.neighbour = ptr(keep[5])
    m.nPatches = len(mesh.patches)
    m.patchStart = ptr(keep[6])
    m.patchSize = ptr(keep[7])
    m.patchLabel = ptr(keep[8])
    m.depth = mesh.depth
    m.periodX, m.periodY = (float(v) for v in mesh.period)
    if mesh.point_alias is not None:
        keep.append(np.ascontiguousarray(mesh.point_alias, dtype=np.int32))
        m.pointAlias = ptr(keep[-1])
    return m, keep


def _cache_key(mesh: FoamMesh, cfg: CaseConfig, Wc, Wb, want_rbf64) -> str:
    h = hashlib.sha256()
    for a in (mesh.points, mesh.cell_ptr, mesh.cell_pts, mesh.face_pts, mesh.owner, mesh.neighbour, Wc,
              np.zeros(0) if Wb is None else Wb, np.zeros(0) if mesh.point_alias is None else mesh.point_alias):
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode() + str(a.shape).encode() + a.tobytes())
    h.update(repr((mesh.patches, mesh.depth, tuple(mesh.period), dataclasses.astuple(cfg), bool(want_rbf64))).encode())
    return h.hexdigest()[:32]


def precompute(mesh: FoamMesh, cfg: CaseConfig, W_cells, W_boundary=None, want_rbf64=False, cache_dir=None,
               device=None, gauss_flux=False):
    """Mesh + initial fields -> the reference's host field bundle (native precompute).

    With ``device`` (a CUDA device index) the RBF stage -- P matrices, inverses, O3 weights -- runs on
    that GPU (``afar_precompute_fields_device``); the bundle is bit-identical to the host's.

    With ``cache_dir`` the bundle is kept on disk under a hash of every input and read back on the
    next call with the same inputs, instead of recomputing the RBF pseudo-inverses and weights (the
    role of the reference's basisOwnList/basisNeiList files and its ``recalcBasis`` switch,
    basicCUDAsolver.cpp:626-694).

    With ``gauss_flux`` the bundle also carries what the optional multi-point face flux needs
    (``afar_precompute_fields_gauss``): ``faceGaussPoints`` (Nf, n, 2), ``faceGaussWeights`` (Nf, n)
    and ``RBFbasisGauss64``, the O3 weights at every point, [face][side][point][maxS+1]."""
    if gauss_flux and cache_dir is not None:
        raise ValueError("precompute: gauss_flux bundles are not cached")
    if cache_dir is not None:
        path = os.path.join(cache_dir, f"afar_bundle_{_cache_key(mesh, cfg, W_cells, W_boundary, want_rbf64)}.npz")
        if os.path.exists(path):
            return HostFields.load(path)
        hf = precompute(mesh, cfg, W_cells, W_boundary, want_rbf64, device=device)
        os.makedirs(cache_dir, exist_ok=True)
        tmp = path + f".{os.getpid()}.tmp.npz"
        hf.save(tmp)
        os.replace(tmp, path)
        return hf
    m, keep = poly_mesh_c(mesh)
    Wc = np.ascontiguousarray(W_cells, dtype=np.float64)
    Wb = None if W_boundary is None else np.ascontiguousarray(W_boundary, dtype=np.float64)
    assert Wc.shape == (mesh.n_cells, 4)
    if Wb is not None:
        assert Wb.shape == (mesh.n_boundary_faces, 4)
    fp = _ffi.FieldPointer()
    sz = _ffi.FieldSizes()
    c = cfg.to_c()
    r64 = C.c_void_p()
    gw, ng = C.c_void_p(), C.c_int()
    if gauss_flux:
        st = lib().afar_precompute_fields_gauss(C.byref(m), C.byref(c), ptr(Wc), ptr(Wb),
                                                -1 if device is None else int(device), C.byref(fp), C.byref(sz),
                                                C.byref(r64) if want_rbf64 else None, C.byref(gw), C.byref(ng))
    elif device is None:
        st = lib().afar_precompute_fields(C.byref(m), C.byref(c), ptr(Wc), ptr(Wb), C.byref(fp), C.byref(sz),
                                          C.byref(r64) if want_rbf64 else None)
    else:
        st = lib().afar_precompute_fields_device(C.byref(m), C.byref(c), ptr(Wc), ptr(Wb), int(device), C.byref(fp),
                                                 C.byref(sz), C.byref(r64) if want_rbf64 else None)
    check(st)
    try:
        hf = HostFields.from_c(fp, sz)
        hf.period = tuple(float(v) for v in mesh.period)
        if want_rbf64:
            n = hf.a["RBFbasis"].shape[0]
            buf = (C.c_double * n).from_address(r64.value) if n else None
            hf.a["RBFbasis64"] = np.frombuffer(buf, dtype=np.float64).copy() if n else np.zeros(0)
        if gauss_flux:
            nf, nmax = hf.nf, hf.sizes["maxStencilSize"] + 1
            cnt = nf * 2 * ng.value * nmax
            buf = (C.c_double * cnt).from_address(gw.value) if cnt else None
            hf.a["RBFbasisGauss64"] = np.frombuffer(buf, dtype=np.float64).copy() if cnt else np.zeros(0)
            pts, w = face_gauss_quadrature(mesh, cfg)
            hf.a["faceGaussPoints"] = np.ascontiguousarray(pts[:nf])
            hf.a["faceGaussWeights"] = np.ascontiguousarray(w[:nf])
    finally:
        lib().afar_free_host_fields(C.byref(fp))
        if want_rbf64 and r64.value:
            C.CDLL(None).free(r64)
        if gw.value:
            C.CDLL(None).free(gw)
    del keep
    return hf


def gauss_quadrature(mesh: FoamMesh, cfg: CaseConfig):
    """Cell and boundary-face Gauss points/weights (CSR over cells then boundary faces)."""
    m, keep = poly_mesh_c(mesh)
    c = cfg.to_c()
    total = C.c_int()
    check(lib().afar_gauss_quadrature(C.byref(m), C.byref(c), None, None, None, C.byref(total)))
    n = mesh.n_cells + mesh.n_boundary_faces
    off = np.zeros(n + 1, dtype=np.int32)
    pts = np.zeros((total.value, 2))
    w = np.zeros(total.value)
    check(lib().afar_gauss_quadrature(C.byref(m), C.byref(c), ptr(off), ptr(pts), ptr(w), C.byref(total)))
    del keep
    return off, pts, w


def face_gauss_quadrature(mesh: FoamMesh, cfg: CaseConfig):
    """Face Gauss points and weights of every face, internal then boundary in face order (the
    d2GaussQuadrature faceGaussPoints / faceGaussWeights layout): points [nFaces, n, 2], weights
    [nFaces, n] (each face's weights sum to |Sf|)."""
    m, keep = poly_mesh_c(mesh)
    c = cfg.to_c()
    n = C.c_int()
    check(lib().afar_face_gauss_quadrature(C.byref(m), C.byref(c), C.byref(n), None, None))
    pts = np.zeros((mesh.n_faces, n.value, 2))
    w = np.zeros((mesh.n_faces, n.value))
    check(lib().afar_face_gauss_quadrature(C.byref(m), C.byref(c), C.byref(n), ptr(pts), ptr(w)))
    del keep
    return pts, w


class CudaSolver:
    """The reference's basicCUDAsolver on libafar (one mesh, one GPU)."""

    def __init__(self, fields: HostFields, cfg: CaseConfig, policy="ref", device=0, period=None, gauss_flux=False):
        self.cfg = cfg
        self.fields = fields
        self.policy = policy
        self.h = C.c_void_p()
        check(lib().afar_solver_create(C.byref(self.h), _ffi.POLICIES[policy], device))
        s = fields.sizes
        self._fp = fields.to_c()
        check(lib().afar_setDeviceFieldData(self.h, C.byref(self._fp), s["cellsNum"], s["facesNum"],
                                            s["totalBoundaryFacesNum"]))
        period = fields.period if period is None else period
        if any(v > 0 for v in period):
            check(lib().afar_set_periodic(self.h, float(period[0]), float(period[1])))
        if policy == "fp64" and "RBFbasis64" in fields.a:
            r = fields.a["RBFbasis64"]
            check(lib().afar_set_rbf_basis64(self.h, ptr(r), r.shape[0]))
        check(lib().afar_setDeviceFieldDataStencil(
            self.h, C.byref(self._fp), s["cellsNum"], s["facesNum"], s["patchesNum"], s["totalBoundaryFacesNum"],
            s["maxStencilSize"], s["maxCompactStencilSize"], s["maxLocalBlockStencilSize"],
            s["maxCompactLocalBlockStencilSize"]))
        check(lib().afar_set_gas(self.h, cfg.R, cfg.Cv))
        if gauss_flux:
            self.set_face_gauss_flux(fields)

    def set_face_gauss_flux(self, fields: HostFields | None = None):
        """The multi-point face flux (afar_set_face_gauss_flux) from a bundle precomputed with
        ``gauss_flux=True``; ``fields=None`` turns it off (the face-centre flux)."""
        if fields is None:
            check(lib().afar_set_face_gauss_flux(self.h, 0, None, None, None))
            return
        pts = np.ascontiguousarray(fields.a["faceGaussPoints"], dtype=np.float64)
        w = np.ascontiguousarray(fields.a["faceGaussWeights"][0] if fields.nf else np.ones(pts.shape[1]))
        rg = np.ascontiguousarray(fields.a["RBFbasisGauss64"], dtype=np.float64)
        check(lib().afar_set_face_gauss_flux(self.h, pts.shape[1], ptr(pts), ptr(w), ptr(rg)))

    # -- reference-shaped calls (basicCUDAsolver.cpp:854-913)
    def set_delta_t(self) -> float:
        dt = C.c_double()
        check(lib().afar_adjustTimeStep(self.h, self.fields.nf, self.cfg.R, self.cfg.Cv, self.cfg.CFL, C.byref(dt)))
        return dt.value

    def evolve(self, dt: float):
        s = self.fields.sizes
        check(lib().afar_GPUevolve(self.h, self.cfg.R, self.cfg.Cv, dt, s["cellsNum"], s["facesNum"],
                                   s["totalBoundaryFacesNum"], s["maxStencilSize"], s["maxCompactStencilSize"],
                                   s["maxLocalBlockStencilSize"], s["maxCompactLocalBlockStencilSize"]))

    def write_field(self):
        """FD (cells + ghosts) and the shock indicator, as copyFieldDataDeviceToHost."""
        out = self.fields.empty_like_outputs(["FD", "shockIndicator"])
        fp = _ffi.FieldPointer()
        fp.FD = ptr(out["FD"])
        fp.shockIndicator = ptr(out["shockIndicator"])
        check(lib().afar_copyFieldDataDeviceToHost(C.byref(fp), self.h, self.fields.nc, self.fields.nb))
        return out["FD"], out["shockIndicator"]

    # -- native extensions
    def run(self, n_steps: int, dt: float = 0.0, cfl: float | None = None, t_end: float = 0.0, wait=True):
        cfl = self.cfg.CFL if cfl is None else cfl
        f = lib().afar_run if wait else lib().afar_run_async
        check(f(self.h, n_steps, dt, cfl, t_end))

    def synchronize(self):
        check(lib().afar_synchronize(self.h))

    def run_timed(self, n_steps: int, dt: float = 0.0, cfl: float | None = None, t_end: float = 0.0) -> float:
        """Device milliseconds of n_steps graph-replayed steps (CUDA events on the solver stream)."""
        cfl = self.cfg.CFL if cfl is None else cfl
        ms = C.c_float()
        check(lib().afar_run_timed(self.h, n_steps, dt, cfl, t_end, C.byref(ms)))
        return ms.value

    def profile_step(self, dt: float = 0.0, cfl: float | None = None):
        """Device ms per kernel kind over one step: reconstruct, bvd, flux, update, bookkeeping."""
        cfl = self.cfg.CFL if cfl is None else cfl
        ms = (C.c_float * 5)()
        check(lib().afar_profile_step(self.h, dt, cfl, ms))
        return dict(zip(["reconstruct", "bvd", "flux", "update", "bookkeeping"], [float(x) for x in ms]))

    def launches_per_step(self) -> int:
        return lib().afar_launches_per_step(self.h)

    def save(self):
        """In-device checkpoint of the state (bit-exact resume with restore())."""
        check(lib().afar_state_snapshot(self.h, 0))

    def restore(self):
        check(lib().afar_state_snapshot(self.h, 1))

    def stream(self) -> int:
        p = C.c_void_p()
        check(lib().afar_get_stream(self.h, C.byref(p)))
        return p.value or 0

    def time(self):
        t, dt, n = C.c_double(), C.c_double(), C.c_longlong()
        check(lib().afar_get_time(self.h, C.byref(t), C.byref(dt), C.byref(n)))
        return t.value, dt.value, n.value

    def set_time(self, t: float):
        check(lib().afar_set_time(self.h, t))

    def state(self):
        out = self.fields.empty_like_outputs(["FD", "cFD", "shockIndicator"])
        check(lib().afar_download_state(self.h, ptr(out["FD"]), ptr(out["cFD"]), ptr(out["shockIndicator"])))
        return out

    def upload_state(self, FD=None, cFD=None, cFDold=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (FD, cFD, cFDold)]
        check(lib().afar_upload_state(self.h, *[ptr(a) for a in arrs]))

    def stage_debug(self, stage: int, dt: float):
        names = ["faceFD", "gradFD", "limiter", "shockIndicator", "Flux", "Res", "FD", "cFD"]
        out = self.fields.empty_like_outputs(names)
        fp = _ffi.FieldPointer()
        for n in names:
            setattr(fp, n, ptr(out[n]))
        check(lib().afar_stage_debug(self.h, stage, dt, C.byref(fp)))
        return out

    def limiter64(self):
        out = np.zeros((self.fields.nc, 4))
        check(lib().afar_debug_limiter64(self.h, ptr(out)))
        return out

    def ls_matrix(self):
        out = np.zeros_like(self.fields.a["matrix"])
        check(lib().afar_download_ls_matrix(self.h, ptr(out)))
        return out

    def set_step_params(self, dt: float = 0.0, cfl: float | None = None, t_end: float = 0.0):
        """Step control used when this solver is stepped inside a Batch (fixed dt, or CFL; t_end clamps)."""
        cfl = self.cfg.CFL if cfl is None else cfl
        check(lib().afar_set_step_params(self.h, dt, cfl, t_end))

    def write_checkpoint(self, path: str):
        """The state on disk for a bit-exact restart: primitive fields with ghosts, conserved fields and
        the simulated time, read between steps.  (The shock flags and the step's intermediates are
        recomputed from these by the next step.)"""
        st = self.state()
        t, last, n = self.time()
        np.savez(path, FD=st["FD"], cFD=st["cFD"], t=np.float64(t), last_dt=np.float64(last), steps=np.int64(n),
                 policy=self.policy, cells=np.int64(self.fields.nc), boundary_faces=np.int64(self.fields.nb))

    def read_checkpoint(self, path: str):
        z = np.load(path)
        if str(z["policy"]) != self.policy or int(z["cells"]) != self.fields.nc or \
                int(z["boundary_faces"]) != self.fields.nb:
            raise ValueError("checkpoint of another mesh or policy")
        self.upload_state(FD=z["FD"], cFD=z["cFD"], cFDold=z["cFD"])
        self.set_time(float(z["t"]))

    def set_tuning(self, recon_variant: int = -1):
        """Mixed reconstruct: -1 autotune, 0 tile-staged, 1 register pass."""
        check(lib().afar_set_tuning(self.h, recon_variant))

    def tuning(self) -> dict:
        v, a, b = C.c_int(), C.c_float(), C.c_float()
        check(lib().afar_get_tuning(self.h, C.byref(v), C.byref(a), C.byref(b)))
        return {"recon_variant": v.value, "ms_tile": a.value, "ms_register": b.value}

    def set_write_interval(self, interval: float):
        """Land graph-replayed steps on multiples of ``interval`` (OpenFOAM adjustableRunTime); 0: off."""
        check(lib().afar_set_write_interval(self.h, interval))

    def switch_counts(self) -> dict:
        """Switch decisions of the last stage: troubled cells, low-order (TVD) cells, shock cells,
        KFVS faces."""
        out = (C.c_longlong * 4)()
        check(lib().afar_switch_counts(self.h, out))
        return dict(zip(["troubled_cells", "tvd_cells", "shock_cells", "kfvs_faces"], [int(v) for v in out]))

    def device_bytes(self) -> int:
        b = C.c_size_t()
        check(lib().afar_device_bytes(self.h, C.byref(b)))
        return b.value

    def close(self):
        if self.h:
            lib().afar_freeFieldData(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several solves (meshes, states, step controls of their own) advanced by one graph of batched
    launches: each kernel's grid covers the blocks of every member.  A member's result is bitwise the
    one it gets when stepped alone.  Members join and leave between runs."""

    def __init__(self, policy="mixed", device=0):
        self.policy = policy
        self.h = C.c_void_p()
        self.members = []
        check(lib().afar_batch_create(C.byref(self.h), _ffi.POLICIES[policy], device))

    def add(self, solver: CudaSolver):
        check(lib().afar_batch_add(self.h, solver.h))
        self.members.append(solver)

    def remove(self, solver: CudaSolver):
        check(lib().afar_batch_remove(self.h, solver.h))
        self.members.remove(solver)

    def __len__(self):
        n = C.c_int()
        check(lib().afar_batch_size(self.h, C.byref(n)))
        return n.value

    def run(self, n_steps: int) -> float:
        """Advance every member n_steps; returns device milliseconds (CUDA events on the batch stream)."""
        ms = C.c_float()
        check(lib().afar_batch_run(self.h, n_steps, C.byref(ms)))
        return ms.value

    def schedule(self) -> dict:
        """The autotuner's launch schedule (afar_batch_get_schedule): members on the tile-staged and
        register-pass reconstruct, BVD and flux block sizes, and the launch times it measured."""
        t, r, bb, fb = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        ms = (C.c_float * 5)()
        check(lib().afar_batch_get_schedule(self.h, C.byref(t), C.byref(r), C.byref(bb), C.byref(fb), ms))
        return {"tile_members": t.value, "register_members": r.value, "bvd_block": bb.value, "flux_block": fb.value,
                "ms_bvd": {64: ms[0], 128: ms[1], 256: ms[2]}, "ms_flux": {128: ms[3], 256: ms[4]}}

    def set_schedule(self, bvd_block: int = 0, flux_block: int = 0):
        """Forces the BVD and flux block sizes (0: autotune)."""
        check(lib().afar_batch_set_schedule(self.h, bvd_block, flux_block))

    def close(self):
        if self.h:
            lib().afar_batch_destroy(self.h)
            self.h = C.c_void_p()
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A queue of solves served on one GPU under a device-memory budget (afar_server_*): requests
    wait until their estimated memory fits beside the running ones, run together as one batch in
    chunks of ``chunk_steps`` steps, and are retired (fields copied out, memory freed) when they
    reach their end time or step count."""

    def __init__(self, policy="mixed", device=0, hbm_budget_bytes=180 << 30, chunk_steps=50):
        self.h = C.c_void_p()
        self._keep = {}
        check(lib().afar_server_create(C.byref(self.h), _ffi.POLICIES[policy], device, int(hbm_budget_bytes),
                                       int(chunk_steps)))
        self.policy = policy

    def submit(self, fields: HostFields, cfg: CaseConfig, t_end: float = 0.0, n_steps: int = 0) -> int:
        fp = fields.to_c()
        out_FD = np.zeros((fields.nc + fields.nb, 4))
        out_si = np.zeros(2 * (fields.nc + fields.nb), dtype=np.int8)
        r = _ffi.Request()
        r.host = C.pointer(fp)
        for k, v in fields.sizes.items():
            setattr(r.sizes, k, int(v))
        r64 = fields.a.get("RBFbasis64") if self.policy == "fp64" else None
        if r64 is not None:
            r.RBFbasis64 = ptr(r64)
            r.RBFbasis64Count = r64.shape[0]
        r.R, r.Cv, r.CFL, r.tEnd, r.nSteps = cfg.R, cfg.Cv, cfg.CFL, t_end, n_steps
        r.outFD = ptr(out_FD)
        r.outShockIndicator = ptr(out_si)
        rid = C.c_longlong()
        check(lib().afar_server_submit(self.h, C.byref(r), C.byref(rid)))
        self._keep[rid.value] = (fields, fp, r, out_FD, out_si)  # alive until the request is done
        return rid.value

    def wait(self, rid: int, timeout: float = -1.0, with_steps: bool = False):
        """(FD, shock indicator, latency ms[, steps]) once the request is done; None on timeout.
        Raises AfarError for a failed request (AFAR_ERR_NOT_FINITE: its state broke down)."""
        done, status, lat, steps = C.c_int(), C.c_int(), C.c_double(), C.c_longlong()
        check(lib().afar_server_wait(self.h, rid, timeout, C.byref(done), C.byref(status), C.byref(lat),
                                     C.byref(steps)))
        if not done.value:
            return None
        _, _, _, out_FD, out_si = self._keep.pop(rid)
        check(status.value)
        return (out_FD, out_si, lat.value, steps.value) if with_steps else (out_FD, out_si, lat.value)

    def cancel(self, rid: int):
        """Cancel a queued or running request; wait() then raises AfarError (AFAR_ERR_CANCELLED)."""
        check(lib().afar_server_cancel(self.h, int(rid)))

    def stats(self) -> dict:
        st = _ffi.ServerStats()
        check(lib().afar_server_get_stats(self.h, C.byref(st)))
        return {n: getattr(st, n) for n, _ in st._fields_}

    def close(self):
        if self.h:
            lib().afar_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
