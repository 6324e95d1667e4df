"""OpenFOAM's binary file format (controlDict ``writeFormat binary``, the setting of the reference's
own cornerFlow case, simulation/cornerFlow/cornerFlow_cuda/system/controlDict:35): the polyMesh,
the fields and the basisOwnList/basisNeiList weight files read and written in binary give the same
arrays as in ascii -- bit for bit, since binary holds the doubles themselves.  No GPU."""
import os
import shutil

import numpy as np
import pytest

from foam_case import write_case


def _mesh_equal(a, b):
    assert np.array_equal(a.points, b.points)
    for k in ("cell_ptr", "cell_pts", "face_pts", "owner", "neighbour"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert a.patches == b.patches and a.depth == b.depth


def test_binary_poly_mesh_reads_like_ascii(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case = foam.load_case(write_case(str(tmp_path / "case"), n=3))
    m = case.mesh
    labels = {0: 3, 1: 4, 2: 2}
    for fmt in ("ascii", "binary"):
        foam.write_poly_mesh(str(tmp_path / fmt), m, binary=fmt == "binary")
    a = foam.read_poly_mesh(str(tmp_path / "ascii"), labels)
    b = foam.read_poly_mesh(str(tmp_path / "binary"), labels)
    _mesh_equal(a, b)
    _mesh_equal(a, m)
    faces = open(tmp_path / "binary" / "constant" / "polyMesh" / "faces", "rb").read()
    assert b"format      binary;" in faces and b"class       faceCompactList;" in faces
    assert b'arch        "LSB;label=32;scalar=64";' in faces


def test_binary_fields_round_trip_bit_exact(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case = foam.load_case(write_case(str(tmp_path / "case"), n=2))
    m = case.mesh
    rng = np.random.default_rng(3)
    FD = rng.uniform(0.5, 2.0, (m.n_cells + m.n_boundary_faces, 4))
    flags = np.zeros(2 * (m.n_cells + m.n_boundary_faces), dtype=np.int8)
    flags[1::2] = rng.integers(-2, 2, flags[1::2].shape[0])
    d = foam.write_fields(str(tmp_path / "out"), 0.005, m, FD, flags, binary=True)
    assert np.array_equal(foam.read_field(os.path.join(d, "p")), FD[:m.n_cells, 0])
    U = foam.read_field(os.path.join(d, "U"))
    assert np.array_equal(U[:, :2], FD[:m.n_cells, 1:3]) and np.all(U[:, 2] == 0)
    assert np.array_equal(foam.read_field(os.path.join(d, "shockIndicator")), flags[1:2 * m.n_cells:2])
    # the patch values are binary lists too: the ghost states come back as written
    fd = foam.read_field_dict(os.path.join(d, "T"))
    off = 0
    for name, _, _, size in m.patches:
        assert np.array_equal(fd["boundaryField"][name]["value"], FD[m.n_cells + off:m.n_cells + off + size, 3])
        off += size


def test_case_with_binary_mesh_and_fields_loads_like_ascii(tmp_path):
    """A case whose constant/polyMesh and 0/ fields are binary (as blockMesh and an OpenFOAM
    utility write them under writeFormat binary) loads to the same mesh, states and ghosts."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    base = write_case(str(tmp_path / "case"), n=2)
    ref = foam.load_case(base, renumber=False)
    m = ref.mesh
    FD = np.concatenate([ref.W, ref.Wb])
    flags = np.zeros(2 * (m.n_cells + m.n_boundary_faces), dtype=np.int8)
    for fmt in ("ascii", "binary"):
        d = str(tmp_path / fmt)
        shutil.copytree(base, d)
        foam.write_poly_mesh(d, m, binary=fmt == "binary")
        # the written fields become the initial fields (time 0)
        out = foam.write_fields(str(tmp_path / (fmt + "_f")), 0.0, m, FD, flags, binary=fmt == "binary")
        for name in ("p", "U", "T"):
            shutil.copy(os.path.join(out, name), os.path.join(d, "0", name))
    a = foam.load_case(str(tmp_path / "ascii"))
    b = foam.load_case(str(tmp_path / "binary"))
    _mesh_equal(a.mesh, b.mesh)
    assert np.allclose(a.W, b.W, rtol=1e-8) and np.allclose(a.Wb, b.Wb, rtol=1e-8)  # ascii keeps 9 digits
    assert np.array_equal(b.W, ref.W) and np.array_equal(b.Wb, ref.Wb)              # binary keeps them all


def test_binary_basis_lists_round_trip(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300.solver import HostFields

    case = foam.load_case(write_case(str(tmp_path / "case"), n=2))
    hf = precompute(case.mesh, case.config, case.W, case.Wb, want_rbf64=True)
    sysd = str(tmp_path / "system")
    foam.write_basis_lists(sysd, hf, binary=True)
    back = HostFields(hf.sizes, {k: (v.copy() if k != "RBFbasis" else np.zeros_like(v)) for k, v in hf.a.items()})
    del back.a["RBFbasis64"]
    foam.read_basis_lists(sysd, back)
    assert np.array_equal(back.a["RBFbasis64"], hf.a["RBFbasis64"])
    assert np.array_equal(back.a["RBFbasis"], hf.a["RBFbasis"])
    # a list of the wrong length is refused
    raw = open(os.path.join(sysd, "basisOwnList"), "rb").read()
    nf = hf.sizes["facesNum"]
    bad = raw.replace(f"\n{nf}\n(".encode(), f"\n{nf + 1}\n(".encode(), 1)
    open(os.path.join(sysd, "basisOwnList"), "wb").write(bad)
    with pytest.raises(ValueError):
        foam.read_basis_lists(sysd, back)


def test_binary_payload_forms(tmp_path):
    """The payload syntax OpenFOAM uses: "N" then "(<bytes>)", 64-bit labels when the header's arch
    says so, an empty list with no parentheses, a truncated payload refused."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    def put(name, body, arch="LSB;label=32;scalar=64"):
        p = tmp_path / name
        p.write_bytes(b'FoamFile\n{\n    format binary;\n    arch "' + arch.encode() + b'";\n    class labelList;\n}\n'
                      + body)
        return str(p)

    lab = np.array([3, 1, 4, 1, 5], dtype="<i8")
    p = put("l64", b"\n5\n(" + lab.tobytes() + b")\n", arch="LSB;label=64;scalar=64")
    assert np.array_equal(foam._read_numbers(p, 1, np.int64), lab)
    p = put("l32", b"\n5\n(" + lab.astype("<i4").tobytes() + b")\n")
    assert np.array_equal(foam._read_numbers(p, 1, np.int64), lab)
    p = put("empty", b"\n0\n\n")
    assert foam._read_numbers(p, 1, np.int64).shape == (0,)
    p = put("short", b"\n5\n(" + lab.astype("<i4").tobytes()[:-3] + b")\n")
    with pytest.raises(ValueError):
        foam._read_numbers(p, 1, np.int64)
    p = put("msb", b"\n0\n", arch="MSB;label=32;scalar=64")
    with pytest.raises(ValueError):
        foam._read_numbers(p, 1, np.int64)
