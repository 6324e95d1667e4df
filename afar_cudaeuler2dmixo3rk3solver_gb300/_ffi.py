"""ctypes declarations of include/afar.h (the C ABI of libafar)."""
from __future__ import annotations

import ctypes as C
import os
import platform

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", platform.machine(), "libafar.so")

AFAR_POLICY_REF = 0
AFAR_POLICY_FP64 = 1
AFAR_POLICY_MIXED = 2
POLICIES = {"ref": AFAR_POLICY_REF, "fp64": AFAR_POLICY_FP64, "mixed": AFAR_POLICY_MIXED}

STENCIL_FACE_NEIGHBOUR = 0
STENCIL_EDGE_NEIGHBOUR = 1

BLOCKDIM = 128

_p = C.c_void_p


class FieldPointer(C.Structure):
    """afar_fieldPointer: the reference's fieldPointer (basicDataStructure.h:75-160)."""
    _fields_ = [(n, _p) for n in (
        "CELL", "FACE", "cellVolume", "FD", "limiter", "shockIndicator", "cFD", "cFDold", "gradFD", "Flux", "Res",
        "neighbour", "boundaryFacesNum", "boundaryFaceNeiLabel", "boundaryFacesType", "stencilSize",
        "compactStencilSize", "RBFbasis", "faceFD", "extendStencil", "extendStencilSize",
        "compactExtendStencilSize", "localStencil", "matrix", "cellFaces", "minDeltaT")]


class FieldSizes(C.Structure):
    _fields_ = [(n, C.c_int) for n in (
        "cellsNum", "facesNum", "patchesNum", "totalBoundaryFacesNum", "maxStencilSize",
        "maxCompactStencilSize", "maxLocalBlockStencilSize", "maxCompactLocalBlockStencilSize")]


class PolyMesh(C.Structure):
    _fields_ = [
        ("nPoints", C.c_int), ("points", _p), ("nCells", C.c_int), ("cellPointsOffset", _p), ("cellPoints", _p),
        ("nInternalFaces", C.c_int), ("nFaces", C.c_int), ("facePoints", _p), ("owner", _p), ("neighbour", _p),
        ("nPatches", C.c_int), ("patchStart", _p), ("patchSize", _p), ("patchLabel", _p), ("depth", C.c_double),
        ("periodX", C.c_double), ("periodY", C.c_double), ("pointAlias", _p),
    ]


class CaseConfig(C.Structure):
    _fields_ = [
        ("R", C.c_double), ("Cv", C.c_double), ("CFL", C.c_double), ("shapeFactor", C.c_double),
        ("stencilType", C.c_int), ("cOrder", C.c_int), ("fOrder", C.c_int), ("nThreads", C.c_int),
    ]


class Request(C.Structure):
    """afar_request: one solve for afar_server_submit."""
    _fields_ = [("host", C.POINTER(FieldPointer)), ("sizes", FieldSizes), ("RBFbasis64", _p),
                ("RBFbasis64Count", C.c_size_t), ("R", C.c_double), ("Cv", C.c_double), ("CFL", C.c_double),
                ("tEnd", C.c_double), ("nSteps", C.c_int), ("outFD", _p), ("outShockIndicator", _p)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("submitted", "completed", "failed", "queued", "running",
                                             "peakRunning")] + [
        ("bytesInUse", C.c_size_t), ("peakBytes", C.c_size_t), ("budgetBytes", C.c_size_t),
        ("batchSteps", C.c_longlong), ("cancelled", C.c_longlong)]


class AfarError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"afar status {status}: {msg}")
        self.status = status


_lib = None


def lib():
    """The loaded libafar.so.  Raises if it has not been built: there is no fallback path."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (the CUDA path has no fallback)")
        L = C.CDLL(LIB_PATH)
        S = C.c_int
        sig = {
            "afar_last_error": (C.c_char_p, []),
            "afar_default_case_config": (None, [C.POINTER(CaseConfig)]),
            "afar_precompute_fields": (S, [C.POINTER(PolyMesh), C.POINTER(CaseConfig), _p, _p,
                                           C.POINTER(FieldPointer), C.POINTER(FieldSizes), C.POINTER(_p)]),
            "afar_free_host_fields": (None, [C.POINTER(FieldPointer)]),
            "afar_precompute_fields_device": (S, [C.POINTER(PolyMesh), C.POINTER(CaseConfig), _p, _p, C.c_int,
                                                  C.POINTER(FieldPointer), C.POINTER(FieldSizes), C.POINTER(_p)]),
            "afar_precompute_fields_gauss": (S, [C.POINTER(PolyMesh), C.POINTER(CaseConfig), _p, _p, C.c_int,
                                                 C.POINTER(FieldPointer), C.POINTER(FieldSizes), C.POINTER(_p),
                                                 C.POINTER(_p), C.POINTER(C.c_int)]),
            "afar_gauss_quadrature": (S, [C.POINTER(PolyMesh), C.POINTER(CaseConfig), _p, _p, _p, C.POINTER(C.c_int)]),
            "afar_face_gauss_quadrature": (S, [C.POINTER(PolyMesh), C.POINTER(CaseConfig), C.POINTER(C.c_int), _p, _p]),
            "afar_solver_create": (S, [C.POINTER(_p), C.c_int, C.c_int]),
            "afar_setDeviceFieldData": (S, [_p, C.POINTER(FieldPointer), C.c_int, C.c_int, C.c_int]),
            "afar_setDeviceFieldDataStencil": (S, [_p, C.POINTER(FieldPointer)] + [C.c_int] * 8),
            "afar_adjustTimeStep": (S, [_p, C.c_int, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]),
            "afar_GPUevolve": (S, [_p, C.c_double, C.c_double, C.c_double] + [C.c_int] * 7),
            "afar_copyFieldDataDeviceToHost": (S, [C.POINTER(FieldPointer), _p, C.c_int, C.c_int]),
            "afar_freeFieldData": (S, [_p]),
            "afar_set_gas": (S, [_p, C.c_double, C.c_double]),
            "afar_set_rbf_basis64": (S, [_p, _p, C.c_size_t]),
            "afar_run": (S, [_p, C.c_int, C.c_double, C.c_double, C.c_double]),
            "afar_run_async": (S, [_p, C.c_int, C.c_double, C.c_double, C.c_double]),
            "afar_synchronize": (S, [_p]),
            "afar_get_stream": (S, [_p, C.POINTER(_p)]),
            "afar_run_timed": (S, [_p, C.c_int, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_float)]),
            "afar_profile_step": (S, [_p, C.c_double, C.c_double, C.POINTER(C.c_float)]),
            "afar_state_snapshot": (S, [_p, C.c_int]),
            "afar_adjustTimeStep_noalloc": (S, [_p, _p, _p, _p, C.c_int, C.c_double, C.c_double, C.c_double, _p,
                                                _p]),
            "afar_get_time": (S, [_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
            "afar_set_time": (S, [_p, C.c_double]),
            "afar_stage_debug": (S, [_p, C.c_int, C.c_double, C.POINTER(FieldPointer)]),
            "afar_debug_limiter64": (S, [_p, _p]),
            "afar_upload_state": (S, [_p, _p, _p, _p]),
            "afar_download_state": (S, [_p, _p, _p, _p]),
            "afar_download_ls_matrix": (S, [_p, _p]),
            "afar_device_bytes": (S, [_p, C.POINTER(C.c_size_t)]),
            "afar_measure_fp64_peak": (S, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_float)]),
            "afar_debug_wait_injection": (S, [C.c_int, C.c_uint, C.c_longlong]),
            "afar_set_face_gauss_flux": (S, [_p, C.c_int, _p, _p, _p]),
            "afar_launches_per_step": (C.c_int, [_p]),
            "afar_set_step_params": (S, [_p, C.c_double, C.c_double, C.c_double]),
            "afar_set_write_interval": (S, [_p, C.c_double]),
            "afar_set_periodic": (S, [_p, C.c_double, C.c_double]),
            "afar_set_tuning": (S, [_p, C.c_int]),
            "afar_get_tuning": (S, [_p, C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "afar_server_create": (S, [C.POINTER(_p), C.c_int, C.c_int, C.c_size_t, C.c_int]),
            "afar_server_submit": (S, [_p, C.POINTER(Request), C.POINTER(C.c_longlong)]),
            "afar_server_wait": (S, [_p, C.c_longlong, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
            "afar_server_get_stats": (S, [_p, C.POINTER(ServerStats)]),
            "afar_server_destroy": (S, [_p]),
            "afar_server_cancel": (S, [_p, C.c_longlong]),
            "afar_switch_counts": (S, [_p, C.POINTER(C.c_longlong)]),
            "afar_batch_create": (S, [C.POINTER(_p), C.c_int, C.c_int]),
            "afar_batch_add": (S, [_p, _p]),
            "afar_batch_remove": (S, [_p, _p]),
            "afar_batch_size": (S, [_p, C.POINTER(C.c_int)]),
            "afar_batch_run": (S, [_p, C.c_int, C.POINTER(C.c_float)]),
            "afar_batch_destroy": (S, [_p]),
            "afar_batch_get_schedule": (S, [_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(C.c_int), C.POINTER(C.c_float)]),
            "afar_batch_set_schedule": (S, [_p, C.c_int, C.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != 0:
        raise AfarError(status, lib().afar_last_error().decode(errors="replace"))


def ptr(a):
    """Data pointer of a numpy array (None for None)."""
    if a is None:
        return None
    assert isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


EXPORTED = [
    "afar_last_error", "afar_default_case_config", "afar_precompute_fields", "afar_free_host_fields",
    "afar_precompute_fields_device",
    "afar_gauss_quadrature", "afar_face_gauss_quadrature", "afar_precompute_fields_gauss", "afar_solver_create", "afar_setDeviceFieldData", "afar_setDeviceFieldDataStencil",
    "afar_adjustTimeStep", "afar_GPUevolve", "afar_copyFieldDataDeviceToHost", "afar_freeFieldData", "afar_set_gas",
    "afar_set_rbf_basis64", "afar_run", "afar_run_async", "afar_synchronize", "afar_get_stream", "afar_get_time",
    "afar_set_time", "afar_stage_debug", "afar_debug_limiter64", "afar_upload_state", "afar_download_state",
    "afar_download_ls_matrix", "afar_device_bytes", "afar_launches_per_step", "afar_run_timed",
    "afar_profile_step", "afar_state_snapshot", "afar_adjustTimeStep_noalloc", "afar_set_step_params",
    "afar_set_write_interval", "afar_set_periodic", "afar_set_tuning", "afar_get_tuning", "afar_batch_create", "afar_batch_add", "afar_batch_remove", "afar_batch_size", "afar_batch_run",
    "afar_batch_destroy", "afar_batch_get_schedule", "afar_batch_set_schedule", "afar_server_create", "afar_server_submit", "afar_server_wait", "afar_server_get_stats",
    "afar_server_destroy", "afar_server_cancel", "afar_switch_counts", "afar_measure_fp64_peak",
    "afar_debug_wait_injection", "afar_set_face_gauss_flux",
]
