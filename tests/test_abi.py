"""The C ABI library loads and exports every entry point include/afar.h declares; error paths
return status codes (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available


def _declared():
    src = open(os.path.join(ROOT, "include", "afar.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(afar_[A-Za-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

    L = C.CDLL(_ffi.LIB_PATH)
    names = _declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(_ffi.EXPORTED) == names


def test_library_is_in_tree():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

    assert os.path.commonpath([_ffi.LIB_PATH, ROOT]) == ROOT


def test_struct_layouts_match_reference():
    """basicDataStructure.h: the POD structs the reference exposes keep their sizes."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

    assert C.sizeof(_ffi.FieldPointer) == 26 * 8
    assert C.sizeof(_ffi.FieldSizes) == 8 * 4


def test_last_error_and_null_arguments():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

    L = _ffi.lib()
    assert L.afar_solver_create(None, 0, 0) == 1
    assert b"null" in L.afar_last_error()
    assert L.afar_solver_create(C.byref(C.c_void_p()), 7, 0) == 1
    assert L.afar_freeFieldData(None) == 0
    assert L.afar_launches_per_step(None) == 13
    # batches: the reference-parity policy is not batched; null arguments are rejected before any CUDA call
    assert L.afar_batch_create(C.byref(C.c_void_p()), 0, 0) == 1
    assert L.afar_batch_create(None, 2, 0) == 1
    assert L.afar_batch_add(None, None) == 1
    assert L.afar_batch_size(None, None) == 1
    assert L.afar_batch_run(None, 1, None) == 1
    assert L.afar_batch_destroy(None) == 0
    assert L.afar_set_step_params(None, 0.0, 0.3, 0.0) != 0


@pytest.mark.skipif(gpu_available(), reason="checks the no-device error path")
def test_no_device_reports_error_not_crash():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

    h = C.c_void_p()
    st = _ffi.lib().afar_solver_create(C.byref(h), 0, 0)
    assert st in (1, 4)
    assert not h.value


def test_precompute_rejects_bad_meshes():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError, CaseConfig, mesh, precompute

    m = mesh.quad_grid(4, 4)
    W, Wb = mesh.uniform_fields(m, 1.0, 0.0, 0.0, 1.0)
    bad = mesh.FoamMesh(**{**m.__dict__})
    bad.face_pts = m.face_pts[:, ::-1].copy()  # normals into the owner
    with pytest.raises(AfarError, match="normal"):
        precompute(bad, CaseConfig(), W, Wb)
    bad = mesh.FoamMesh(**{**m.__dict__})
    bad.neighbour = m.neighbour.copy()
    bad.neighbour[0] = m.owner[0]  # owner == neighbour
    with pytest.raises(AfarError):
        precompute(bad, CaseConfig(), W, Wb)
    with pytest.raises(AfarError, match="stencil type"):
        precompute(m, CaseConfig(stencilType="faceNeighbour") if False else _bad_cfg(), W, Wb)


def _bad_cfg():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig

    c = CaseConfig()
    c.to_c_orig = c.to_c

    def to_c():
        s = c.to_c_orig()
        s.stencilType = 5
        return s

    c.to_c = to_c
    return c


def test_stencil_limit_is_enforced():
    """MAX_VALID_STENCIL_SIZE (basicDataStructure.h:8): a fan of 24 triangles around one vertex
    gives a 25-cell vertex neighbourhood, which the reference rejects."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError, CaseConfig, mesh, precompute

    n = 24
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    pts = np.concatenate([[[0.0, 0.0]], np.stack([np.cos(ang), np.sin(ang)], 1)])
    tris = np.array([[0, 1 + i, 1 + (i + 1) % n] for i in range(n)])
    m = mesh.build_foam_mesh(pts, np.arange(0, 3 * n + 1, 3), tris.ravel(), lambda x, y: np.zeros(x.shape[0], int),
                             [("wall", 2)], renumber=False)
    W, Wb = mesh.uniform_fields(m, 1.0, 0.0, 0.0, 1.0)
    with pytest.raises(AfarError, match="Too large stencil"):
        precompute(m, CaseConfig(stencilType="edgeNeighbour"), W, Wb)
    hf = precompute(m, CaseConfig(stencilType="faceNeighbour"), W, Wb)
    assert hf.sizes["maxStencilSize"] <= 20


def test_server_rejects_bad_arguments_without_a_gpu():
    import ctypes as C

    from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

    L = _ffi.lib()
    h = C.c_void_p()
    assert L.afar_server_create(C.byref(h), 0, 0, 1 << 30, 50) == 1  # the ref policy is not served
    assert L.afar_server_create(C.byref(h), 2, 0, 1 << 30, 0) == 1   # chunk of 0 steps
    assert L.afar_server_submit(None, None, None) == 1
    assert L.afar_server_get_stats(None, None) == 1
    assert L.afar_server_destroy(None) == 0
    assert L.afar_server_cancel(None, 1) == 1
