"""OpenFOAM case handling (no GPU): dictionary parsing, the 2-D blockMesh, the initial fields and
the OpenFOAM ascii writers."""
import os

import numpy as np
import pytest

from conftest import ROOT
from foam_case import write_case
from oracle.reference_dir import reference_dir


def test_parse_dictionary_forms():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    d = foam.parse_foam("""/* block */ a 1; b 2.5e-3; // line
    c { d word; e (1 2 (3 4)); } f uniform (4.5 0 0); g [0 1 -1 0 0 0 0]; h "quoted text";""")
    assert d["a"] == 1 and d["b"] == 2.5e-3
    assert d["c"]["d"] == "word" and d["c"]["e"] == [1, 2, [3, 4]]
    assert d["f"] == ["uniform", [4.5, 0, 0]]
    assert d["g"] == [0, 1, -1, 0, 0, 0, 0] and d["h"] == "quoted text"
    with pytest.raises(ValueError):
        foam.parse_foam("#include \"other\"")


def test_forward_step_case_mesh_and_fields(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam, precompute

    case = foam.load_case(write_case(str(tmp_path), n=2))
    m = case.mesh
    assert m.n_cells == 6 * 2 + 6 * 8 + 24 * 8
    names = [p[0] for p in m.patches]
    labels = {p[0]: p[1] for p in m.patches}
    sizes = {p[0]: p[3] for p in m.patches}
    assert names == ["inflow", "outflow", "walls"] and labels == {"inflow": 3, "outflow": 4, "walls": 2}
    assert sizes == {"inflow": 2 + 8, "outflow": 8, "walls": 6 + 2 + 24 + 6 + 24}
    assert np.isclose(m.cell_areas().sum(), 3.0 - 2.4 * 0.2)
    assert case.config.cOrder == 5 and case.config.fOrder == 4 and case.config.CFL == 0.2
    assert case.adjust_time_step and case.end_time == 0.02 and case.write_interval == 0.005
    assert np.allclose(case.W, [1.0, 3.0, 0.0, 1.0])
    # OpenFOAM's initial patch values: slip walls keep the owner's tangential velocity, so the
    # step's vertical face (normal -x) starts at rest; every other ghost is the free stream
    fc = m.boundary_face_centres()
    riser = np.isclose(fc[:, 0], 0.6) & (fc[:, 1] < 0.2)
    assert riser.sum() == 2
    assert np.allclose(case.Wb[riser], [1.0, 0.0, 0.0, 1.0])
    assert np.allclose(case.Wb[~riser], [1.0, 3.0, 0.0, 1.0])
    hf = precompute(m, case.config, case.W, case.Wb)  # the native precompute accepts the mesh
    assert hf.nc == m.n_cells


def test_grading_and_orientation(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    x = foam._grading(4, 8.0)
    d = np.diff(x)
    assert np.isclose(x[-1], 1.0) and np.isclose(d[-1] / d[0], 8.0)
    m = foam.load_case(write_case(str(tmp_path), n=1)).mesh
    assert (m.cell_areas() > 0).all()


def test_writers_round_trip(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case = foam.load_case(write_case(str(tmp_path / "case"), n=2))
    m = case.mesh
    out = str(tmp_path / "out")
    foam.write_poly_mesh(out, m)
    rng = np.random.default_rng(2)
    FD = rng.uniform(0.5, 2.0, (m.n_cells + m.n_boundary_faces, 4))
    flags = np.zeros(2 * (m.n_cells + m.n_boundary_faces), dtype=np.int8)
    flags[1::2] = rng.integers(-2, 2, flags[1::2].shape[0])
    d = foam.write_fields(out, 0.005, m, FD, flags)
    assert os.path.basename(d) == "0.005"
    assert np.allclose(foam.read_field(os.path.join(d, "p")), FD[:m.n_cells, 0], rtol=1e-8)
    U = foam.read_field(os.path.join(d, "U"))
    assert np.allclose(U[:, :2], FD[:m.n_cells, 1:3], rtol=1e-8) and np.all(U[:, 2] == 0)
    assert np.array_equal(foam.read_field(os.path.join(d, "shockIndicator")), flags[1:2 * m.n_cells:2])
    faces = foam.read_foam(os.path.join(out, "constant", "polyMesh", "boundary"))
    poly = os.path.join(out, "constant", "polyMesh")
    owner = open(os.path.join(poly, "owner")).read()
    assert f"\n{m.n_faces + 2 * m.n_cells}\n(" in owner
    assert "defaultFaces" in open(os.path.join(poly, "boundary")).read() and faces is not None


REF_CASE = os.path.join(reference_dir(), "simulation", "cornerFlow", "cornerFlow_cuda")


@pytest.mark.skipif(not os.path.isdir(REF_CASE), reason="the reference's case files are not on this machine")
def test_reference_corner_flow_case_loads():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case = foam.load_case(REF_CASE)
    m = case.mesh
    assert m.n_cells == 250000
    assert [(p[0], p[1], p[3]) for p in m.patches] == [("inlet", 5, 250), ("obstacle", 2, 1250), ("outlet", 4, 500)]
    assert case.config.cOrder == 7 and case.config.fOrder == 5 and case.config.stencilType == "edgeNeighbour"
    assert case.end_time == 0.15 and case.write_interval == 0.01 and case.max_co == 0.3


def test_basis_lists_round_trip(tmp_path):
    """basisOwnList/basisNeiList (basicCUDAsolver.cpp:538-694): written with 17 digits and read
    back, the weights are bit-identical in double and float; one list per internal face with the
    stencil's length."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300.solver import HostFields

    case = foam.load_case(write_case(str(tmp_path / "case"), n=2))
    hf = precompute(case.mesh, case.config, case.W, case.Wb, want_rbf64=True)
    sysd = str(tmp_path / "system")
    foam.write_basis_lists(sysd, hf)
    nf = hf.sizes["facesNum"]
    own = open(os.path.join(sysd, "basisOwnList")).read()
    assert "class       scalarListList;" in own and f"\n{nf}\n(\n" in own
    back = HostFields(hf.sizes, {k: (v.copy() if k != "RBFbasis" else np.zeros_like(v)) for k, v in hf.a.items()})
    del back.a["RBFbasis64"]
    foam.read_basis_lists(sysd, back)
    assert np.array_equal(back.a["RBFbasis64"], hf.a["RBFbasis64"])
    assert np.array_equal(back.a["RBFbasis"], hf.a["RBFbasis"])
    assert back.a["RBFbasis"].dtype == np.float32


def test_basis_lists_openfoam_long_list_form_and_errors(tmp_path):
    """OpenFOAM writes inner lists longer than ten one value per line; both forms read the same.
    A list count or a list length that does not match the mesh's stencils is an error."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam, precompute

    case = foam.load_case(write_case(str(tmp_path / "case"), n=2))
    hf = precompute(case.mesh, case.config, case.W, case.Wb, want_rbf64=True)
    sysd = str(tmp_path / "system")
    foam.write_basis_lists(sysd, hf)
    ref = hf.a["RBFbasis64"].copy()
    path = os.path.join(sysd, "basisNeiList")
    lines = open(path).read().split("\n")
    long = []
    for ln in lines:
        m = __import__("re").match(r"^(\d+)\((.*)\)$", ln)
        if m:
            long += [m.group(1), "("] + m.group(2).split() + [")"]
        else:
            long.append(ln)
    open(path, "w").write("\n".join(long))
    foam.read_basis_lists(sysd, hf)
    assert np.array_equal(hf.a["RBFbasis64"], ref)
    txt = open(os.path.join(sysd, "basisOwnList")).read()
    n0 = int(__import__("re").search(r"\n(\d+)\(", txt).group(1))
    bad = txt.replace(f"\n{n0}(", f"\n{n0 + 1}(0 ", 1)
    open(os.path.join(sysd, "basisOwnList"), "w").write(bad)
    with pytest.raises(ValueError, match="face 0"):
        foam.read_basis_lists(sysd, hf)
    nf = hf.sizes["facesNum"]
    open(os.path.join(sysd, "basisOwnList"), "w").write(txt.replace(f"\n{nf}\n(", f"\n{nf - 1}\n(", 1))
    with pytest.raises(ValueError, match="internal faces"):
        foam.read_basis_lists(sysd, hf)


def test_recalc_basis_switch(tmp_path):
    """fvSchemes CUDA recalcBasis: absent or true computes the weights; false reads them from the
    case's system directory and fails without the files."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam, precompute

    assert foam.load_case(write_case(str(tmp_path / "a"), n=1)).recalc_basis
    case = foam.load_case(write_case(str(tmp_path / "b"), n=1, recalc_basis=False))
    assert not case.recalc_basis
    hf = precompute(case.mesh, case.config, case.W, case.Wb)
    with pytest.raises(FileNotFoundError):
        foam.read_basis_lists(str(tmp_path / "b" / "system"), hf)
