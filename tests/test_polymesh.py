"""Reading an OpenFOAM polyMesh (no GPU): the 2-D cross-section of a one-cell-deep mesh, patch
labels by boundary-file index, nonuniform initial fields, renumbering."""
import os
import re
import shutil

import numpy as np
import pytest

from foam_case import write_case


def _written(tmp_path, n=2):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case = foam.load_case(write_case(str(tmp_path / "case"), n=n))
    out = str(tmp_path / "poly")
    foam.write_poly_mesh(out, case.mesh)
    return case, out


def _same_mesh(a, b):
    for k in ("points", "cell_ptr", "cell_pts", "face_pts", "owner", "neighbour"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert a.patches == b.patches and a.depth == b.depth


def test_poly_mesh_round_trip(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case, out = _written(tmp_path)
    m = foam.read_poly_mesh(out, {0: 3, 1: 4, 2: 2})
    _same_mesh(case.mesh, m)


def test_poly_mesh_openfoam_layouts(tmp_path):
    """Side faces starting at another vertex (same cycle, same normal), the empty patch listed
    first, patches in any order of the boundary file: the same 2-D mesh."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case, out = _written(tmp_path)
    d = os.path.join(out, "constant", "polyMesh")
    txt = open(os.path.join(d, "faces")).read()
    # rotate every side quad "4(a b b' a')" to "4(b b' a' a)" (front and back polygons unchanged)
    npt = case.mesh.points.shape[0]

    def rot(m):
        v = [int(m[k]) for k in range(1, 5)]
        if sum(x < npt for x in v) != 2:
            return m[0]
        return f"\n4({v[1]} {v[2]} {v[3]} {v[0]})"

    txt = re.sub(r"\n4\((\d+) (\d+) (\d+) (\d+)\)", rot, txt)
    open(os.path.join(d, "faces"), "w").write(txt)
    bnd = open(os.path.join(d, "boundary")).read()
    blocks = re.findall(r"    \S+\n    \{[^}]*\}\n", bnd)
    assert len(blocks) == 4
    head = bnd[:bnd.index(blocks[0])]
    open(os.path.join(d, "boundary"), "w").write(head + blocks[3] + "".join(blocks[:3]) + ")\n")
    m = foam.read_poly_mesh(out, {1: 3, 2: 4, 3: 2})  # the empty patch is patch0 now
    _same_mesh(case.mesh, m)


def test_poly_mesh_errors(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    _, out = _written(tmp_path)
    with pytest.raises(ValueError, match="patch2"):
        foam.read_poly_mesh(out, {0: 3, 1: 4})
    d = os.path.join(out, "constant", "polyMesh")
    pts = open(os.path.join(d, "points")).read()
    bad, k = re.subn(r"\((\S+) (\S+) 0\.0\)\n", r"(\1 \2 0.05)\n", pts, count=1)  # off both planes
    assert k == 1
    open(os.path.join(d, "points"), "w").write(bad)
    with pytest.raises(ValueError, match="one-cell-deep"):
        foam.read_poly_mesh(out, {0: 3, 1: 4, 2: 2})


def test_poly_mesh_case_with_nonuniform_fields(tmp_path):
    """A case holding constant/polyMesh loads it instead of meshing blockMeshDict, and reads
    nonuniform initial fields (here the fields written at a time, copied to 0/)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case, out = _written(tmp_path)
    m = case.mesh
    rng = np.random.default_rng(3)
    FD = np.concatenate([case.W, case.Wb]) * (1 + 0.1 * rng.random((m.n_cells + m.n_boundary_faces, 4)))
    flags = np.zeros(2 * (m.n_cells + m.n_boundary_faces), dtype=np.int8)
    tdir = foam.write_fields(out, 0.5, m, FD, flags)
    os.makedirs(os.path.join(out, "system"), exist_ok=True)
    for f in ("fvSchemes", "controlDict"):
        shutil.copy(os.path.join(str(tmp_path / "case"), "system", f), os.path.join(out, "system", f))
    os.makedirs(os.path.join(out, "0"))
    for f in ("p", "U", "T"):
        shutil.copy(os.path.join(tdir, f), os.path.join(out, "0", f))
    back = foam.load_case(out)
    _same_mesh(m, back.mesh)
    assert np.allclose(back.W, FD[:m.n_cells], rtol=1e-8, atol=0)
    # the written boundary values are `calculated` with a value: they come back as written
    assert np.allclose(back.Wb, FD[m.n_cells:], rtol=1e-8, atol=0)


def test_renumber_mesh(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, foam, mesh, precompute

    base = mesh.quad_grid(12, 7, renumber=False)
    r = mesh.renumber_mesh(base)
    assert np.allclose(np.sort(base.cell_areas()), np.sort(r.cell_areas()))
    own, nei = r.owner[:r.n_internal_faces], r.neighbour
    assert np.all(own < nei)
    key = own.astype(np.int64) * r.n_cells + nei
    assert np.all(np.diff(key) > 0)
    # normals still leave the owner: the owner's centroid lies behind every face
    c = r.cell_centres()
    p = r.points
    a, b = p[r.face_pts[:, 0]], p[r.face_pts[:, 1]]
    n = np.stack([b[:, 1] - a[:, 1], a[:, 0] - b[:, 0]], 1)
    assert np.all(np.sum((0.5 * (a + b) - c[r.owner]) * n, 1) > 0)
    W, Wb = mesh.uniform_fields(r, 1.0, 0.5, 0.0, 1.0)
    hf = precompute(r, CaseConfig(), W, Wb)
    assert hf.nc == r.n_cells
    bw = max(abs(int(x) - int(y)) for x, y in zip(own, nei))
    bw0 = max(abs(int(x) - int(y)) for x, y in zip(base.owner[:base.n_internal_faces], base.neighbour))
    assert bw <= bw0


def test_hilbert_order():
    """The Hilbert-curve cell order: a permutation whose consecutive cells are grid neighbours on a
    2^k grid, and a renumbered mesh with the same cells, upper-triangular faces and outward normals,
    whose 128-cell tiles reach fewer stencil cells than reverse Cuthill-McKee's strips."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300.mesh import _hilbert_permutation

    k = 4
    X, Y = np.meshgrid(np.arange(1 << k), np.arange(1 << k), indexing="ij")
    xy = np.stack([X.ravel(), Y.ravel()], 1) + 0.5
    p = _hilbert_permutation(xy, bits=k)
    assert np.array_equal(np.sort(p), np.arange(xy.shape[0]))
    assert np.all(np.abs(np.diff(xy[p], axis=0)).sum(1) == 1.0)

    base = mesh.quad_grid(40, 40, renumber=False, jitter=0.2, seed=3)
    h = mesh.renumber_mesh(base, order="hilbert")
    assert np.allclose(np.sort(base.cell_areas()), np.sort(h.cell_areas()))
    own, nei = h.owner[:h.n_internal_faces], h.neighbour
    assert np.all(np.diff(own.astype(np.int64) * h.n_cells + nei) > 0)
    c = h.cell_centres()
    a, b = h.points[h.face_pts[:, 0]], h.points[h.face_pts[:, 1]]
    n = np.stack([b[:, 1] - a[:, 1], a[:, 0] - b[:, 0]], 1)
    assert np.all(np.sum((0.5 * (a + b) - c[h.owner]) * n, 1) > 0)
    with pytest.raises(ValueError):
        mesh.renumber_mesh(base, order="morton")

    halo = {}
    for order in ("rcm", "hilbert"):
        m = mesh.forward_step_triangles(20000, seed=1, renumber=order)
        W, Wb = mesh.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
        hf = precompute(m, CaseConfig(), W, Wb)
        halo[order] = float(hf.extendStencilSize.astype(np.int64).mean())
    assert halo["hilbert"] < 0.5 * halo["rcm"]
