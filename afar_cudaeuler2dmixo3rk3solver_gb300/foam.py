"""OpenFOAM case files for the AFAR solver: reading the dictionaries a reference case holds, a 2-D
blockMesh, and writing the fields (and the mesh) back in OpenFOAM's ascii format.

The reference application reads an OpenFOAM case: ``system/blockMeshDict`` (meshed by blockMesh),
``system/controlDict`` (end time, write interval, Courant number), ``system/fvSchemes`` (the
``CUDA`` dictionary: gas constants, stencil type and the cudaEulerBCs label of each patch; the
``gaussQuadrature`` orders) and the initial fields ``0/p``, ``0/U``, ``0/T``
(reference ``applications/solvers/compressible/CUDA/cudaEuler2DmixO3RK3solver/
cudaEuler2DmixO3RK3solver.cpp:14-60``, ``src/CUDA/cudaEuler2DmixO3RK3/basicCUDAsolver.cpp:55-68,
122-258, 874-913``).  This module turns such a case into the arrays the solver takes and writes
``p``, ``U``, ``T`` and ``shockIndicator`` per write time, plus ``constant/polyMesh`` so that the
output opens in OpenFOAM tools.  Host-side utility code: no GPU work here.
"""
from __future__ import annotations

import dataclasses
import math
import os
import re

import numpy as np

from . import mesh as M

# ----------------------------------------------------------------------------------- dictionaries
_TOKEN = re.compile(r'"[^"]*"|[{}()\[\];]|[^\s{}()\[\];"]+')


def _strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _atom(tok: str):
    if tok.startswith('"'):
        return tok[1:-1]
    try:
        return int(tok)
    except ValueError:
        pass
    try:
        return float(tok)
    except ValueError:
        return tok


class FoamDict(dict):
    """An OpenFOAM dictionary: keys in file order; a value is a scalar, a word, a list, a
    FoamDict, or (for entries of several items, e.g. ``uniform (1 0 0)``) a list of them."""


def _parse_list(toks, i, close):
    out = []
    while True:
        if i >= len(toks):
            raise ValueError("unterminated list")
        t = toks[i]
        if t == close:
            return out, i + 1
        if t in ("(", "["):
            v, i = _parse_list(toks, i + 1, ")" if t == "(" else "]")
            out.append(v)
        elif t == "{":
            v, i = _parse_dict(toks, i + 1, "}")
            out.append(v)
        elif t == ";":
            i += 1
        else:
            out.append(_atom(t))
            i += 1


def _parse_dict(toks, i, close):
    d = FoamDict()
    while i < len(toks):
        t = toks[i]
        if t == close:
            return d, i + 1
        if t.startswith("#"):
            raise ValueError(f"directive {t} is not supported")
        key = _atom(t)
        i += 1
        if i < len(toks) and toks[i] == "{":
            d[key], i = _parse_dict(toks, i + 1, "}")
            continue
        items = []
        while i < len(toks) and toks[i] != ";":
            if toks[i] in ("(", "["):
                v, i = _parse_list(toks, i + 1, ")" if toks[i] == "(" else "]")
                items.append(v)
            elif toks[i] == "{":
                raise ValueError(f"unexpected '{{' in the entry {key}")
            else:
                items.append(_atom(toks[i]))
                i += 1
        i += 1  # ';'
        d[key] = items[0] if len(items) == 1 else items
    if close != "":
        raise ValueError("unterminated dictionary")
    return d, i


def parse_foam(text: str) -> FoamDict:
    """Parse an OpenFOAM dictionary file (comments, nested dictionaries, lists, ``[dimensions]``)."""
    toks = _TOKEN.findall(_strip_comments(text))
    d, _ = _parse_dict(toks, 0, "")
    return d


def read_foam(path: str) -> FoamDict:
    with open(path) as f:
        return parse_foam(f.read())


# ----------------------------------------------------------------------------------- blockMesh (2-D)
def _grading(n: int, ratio: float) -> np.ndarray:
    """Node positions in [0, 1] for n cells whose last/first size ratio is ``ratio`` (simpleGrading)."""
    if n < 1:
        raise ValueError("a block needs at least one cell per direction")
    if abs(ratio - 1.0) < 1e-12 or n == 1:
        return np.linspace(0.0, 1.0, n + 1)
    q = ratio ** (1.0 / (n - 1))
    sizes = q ** np.arange(n)
    x = np.concatenate([[0.0], np.cumsum(sizes)])
    return x / x[-1]


def block_mesh_2d(bmd: FoamDict, labels: dict, renumber: bool = True) -> M.FoamMesh:
    """Mesh the x-y cross-section of a one-cell-deep blockMeshDict: hex blocks with straight edges
    and simpleGrading, merged at shared nodes.  ``labels`` maps each patch name to its cudaEulerBCs
    label.  Patch faces are matched to boundary edges geometrically; every boundary edge must belong
    to one named patch (front and back are the empty defaultPatch)."""
    scale = float(bmd.get("convertToMeters", bmd.get("scale", 1.0)))
    verts = np.asarray(bmd["vertices"], dtype=np.float64) * scale
    if bmd.get("edges"):
        raise ValueError("curved block edges are not supported")
    blocks = bmd["blocks"]
    z0 = verts[:, 2].min()
    key_scale = 1e-9 * max(1.0, float(np.abs(verts[:, :2]).max()))
    node_of = {}
    pts = []
    quads = []
    i = 0
    while i < len(blocks):
        if blocks[i] != "hex":
            raise ValueError(f"block shape {blocks[i]} is not supported (hex only)")
        ids = [int(v) for v in blocks[i + 1]]
        n = [int(v) for v in blocks[i + 2]]
        i += 3
        grad = [1.0, 1.0, 1.0]
        if i < len(blocks) and blocks[i] == "simpleGrading":
            g = blocks[i + 1]
            if any(isinstance(v, list) for v in g):
                raise ValueError("multi-grading is not supported")
            grad = [float(v) for v in g]
            i += 2
        if n[2] != 1:
            raise ValueError("a 2-D case has one cell in the third direction")
        bot = [v for v in ids[:4]]
        if not np.allclose(verts[bot, 2], z0):
            raise ValueError("the first four vertices of a block must lie on the lower z plane")
        c = verts[bot, :2]
        s = _grading(n[0], grad[0])
        t = _grading(n[1], grad[1])
        S, T = np.meshgrid(s, t, indexing="ij")
        P = ((1 - S)[..., None] * (1 - T)[..., None] * c[0] + S[..., None] * (1 - T)[..., None] * c[1]
             + S[..., None] * T[..., None] * c[2] + (1 - S)[..., None] * T[..., None] * c[3])
        ids_grid = np.empty(S.shape, dtype=np.int64)
        for a in range(S.shape[0]):
            for b in range(S.shape[1]):
                k = (round(P[a, b, 0] / key_scale), round(P[a, b, 1] / key_scale))
                if k not in node_of:
                    node_of[k] = len(pts)
                    pts.append(P[a, b])
                ids_grid[a, b] = node_of[k]
        q = np.stack([ids_grid[:-1, :-1], ids_grid[1:, :-1], ids_grid[1:, 1:], ids_grid[:-1, 1:]], axis=-1).reshape(-1, 4)
        quads.append(q)
    points = np.asarray(pts)
    quads = np.concatenate(quads)
    a, b, c2 = points[quads[:, 0]], points[quads[:, 1]], points[quads[:, 2]]
    area = (b[:, 0] - a[:, 0]) * (c2[:, 1] - a[:, 1]) - (c2[:, 0] - a[:, 0]) * (b[:, 1] - a[:, 1])
    quads[area < 0] = quads[area < 0][:, ::-1]  # counter-clockwise
    # patch edges of the lower plane
    segs, pidx, patch_defs = [], [], []
    bnd = bmd.get("boundary", [])
    names = [bnd[k] for k in range(0, len(bnd), 2)]
    for p, name in enumerate(names):
        spec = bnd[2 * names.index(name) + 1]
        if name not in labels:
            raise ValueError(f"patch {name} has no cudaEulerBCs label")
        patch_defs.append((name, int(labels[name])))
        for face in spec.get("faces", []):
            low = [int(v) for v in face if abs(verts[int(v), 2] - z0) < 1e-12]
            if len(low) != 2:
                raise ValueError(f"patch {name}: face {face} is not a side face of the 2-D mesh")
            segs.append((verts[low[0], :2], verts[low[1], :2]))
            pidx.append(p)
    seg_a = np.asarray([s_[0] for s_ in segs])
    seg_b = np.asarray([s_[1] for s_ in segs])
    pidx = np.asarray(pidx)
    tol = 1e-8 * max(1.0, float(np.abs(points).max()))

    def classify(xm, ym):
        m_ = np.stack([xm, ym], axis=1)
        out = np.full(xm.shape[0], -1, dtype=np.int64)
        for k in range(seg_a.shape[0]):
            d = seg_b[k] - seg_a[k]
            L2 = float(d @ d)
            tpar = ((m_ - seg_a[k]) @ d) / L2
            dist = np.abs((m_[:, 0] - seg_a[k, 0]) * d[1] - (m_[:, 1] - seg_a[k, 1]) * d[0]) / math.sqrt(L2)
            hit = (tpar >= -1e-12) & (tpar <= 1 + 1e-12) & (dist < tol) & (out < 0)
            out[hit] = pidx[k]
        if (out < 0).any():
            raise ValueError(f"{int((out < 0).sum())} boundary edges belong to no patch")
        return out

    cell_ptr = np.arange(0, 4 * quads.shape[0] + 1, 4)
    depth = float(verts[:, 2].max() - z0)
    return M.build_foam_mesh(points, cell_ptr, quads.ravel(), classify, patch_defs, renumber=renumber,
                             depth=depth if depth > 0 else 1.0)


# ----------------------------------------------------------------------------------- the case
@dataclasses.dataclass
class FoamCase:
    mesh: M.FoamMesh
    config: "object"          # CaseConfig
    W: np.ndarray             # (Nc, 4) initial (p, Ux, Uy, T)
    Wb: np.ndarray            # (Nb, 4) initial ghost states
    end_time: float
    write_interval: float
    delta_t: float
    adjust_time_step: bool
    max_co: float
    recalc_basis: bool = True  # fvSchemes CUDA recalcBasis: false reads system/basis{Own,Nei}List


def _uniform(v):
    if isinstance(v, list) and len(v) == 2 and v[0] == "uniform":
        return v[1]
    raise ValueError(f"only uniform values are supported, got {v!r}")


def _field_values(fdict, patches, n_cells, is_vector):
    internal = _uniform(fdict["internalField"])
    nb = sum(p[3] for p in patches)
    cells = np.tile(np.asarray(internal, dtype=np.float64)[:2] if is_vector else [float(internal)], (n_cells, 1))
    ghosts = np.tile(cells[0], (nb, 1))
    bf = fdict.get("boundaryField", {})
    off = 0
    for name, _, _, size in patches:
        spec = bf.get(name, {})
        if spec.get("type") == "fixedValue":
            v = _uniform(spec["value"])
            ghosts[off:off + size] = np.asarray(v, dtype=np.float64)[:2] if is_vector else float(v)
        off += size
    return cells, ghosts


def load_case(case_dir: str, renumber: bool = True) -> FoamCase:
    """The reference case in ``case_dir`` as solver inputs: the meshed cross-section, the case
    configuration (fvSchemes ``CUDA`` and ``gaussQuadrature``, controlDict ``maxCo``), the initial
    cell states and ghost states, and the time controls."""
    from .solver import CaseConfig

    sysd = os.path.join(case_dir, "system")
    schemes = read_foam(os.path.join(sysd, "fvSchemes"))
    control = read_foam(os.path.join(sysd, "controlDict"))
    bmd = read_foam(os.path.join(sysd, "blockMeshDict"))
    cuda = schemes["CUDA"]
    gq = schemes.get("gaussQuadrature", {})
    bnd = bmd.get("boundary", [])
    names = [bnd[k] for k in range(0, len(bnd), 2)]
    blabels = cuda.get("boundary", {})
    labels = {name: int(blabels[f"patch{k}"]) for k, name in enumerate(names) if f"patch{k}" in blabels}
    m = block_mesh_2d(bmd, labels, renumber=renumber)
    max_co = float(control.get("maxCo", 0.5))
    cfg = CaseConfig(R=float(cuda["R"]), Cv=float(cuda["Cv"]), CFL=max_co,
                     stencilType=str(cuda.get("stencilType", "edgeNeighbour")),
                     shapeFactor=float(schemes.get("shapeFactor", 10.0)),
                     cOrder=int(gq.get("cOrder", 5)), fOrder=int(gq.get("fOrder", 4)))
    zero = os.path.join(case_dir, "0")
    p, pb = _field_values(read_foam(os.path.join(zero, "p")), m.patches, m.n_cells, False)
    U, Ub = _field_values(read_foam(os.path.join(zero, "U")), m.patches, m.n_cells, True)
    T, Tb = _field_values(read_foam(os.path.join(zero, "T")), m.patches, m.n_cells, False)
    W = np.concatenate([p, U, T], axis=1)
    Wb = np.concatenate([pb, Ub, Tb], axis=1)
    return FoamCase(mesh=m, config=cfg, W=W, Wb=Wb, end_time=float(control["endTime"]),
                    write_interval=float(control.get("writeInterval", control["endTime"])),
                    delta_t=float(control.get("deltaT", 0.0)),
                    adjust_time_step=str(control.get("adjustTimeStep", "no")) in ("true", "yes", "on", "1"),
                    max_co=max_co, recalc_basis=_truth(cuda.get("recalcBasis", "true")))


def _truth(v) -> bool:
    return str(v) in ("true", "yes", "on", "1")


# ----------------------------------------------------------------------------------- writing
def _header(cls, obj, location=None):
    loc = f'    location    "{location}";\n' if location is not None else ""
    return ("FoamFile\n{\n    version     2.0;\n    format      ascii;\n"
            f"    class       {cls};\n{loc}    object      {obj};\n}}\n\n")


def _fmt(v):
    return f"{v:.9g}"


def write_poly_mesh(out_dir: str, m: M.FoamMesh):
    """``constant/polyMesh`` of the one-cell-deep 3-D mesh: points on z = 0 and z = depth, a quad
    per 2-D face (internal faces first, then the named patches), and the front and back polygons
    of every cell in the empty patch ``defaultFaces``."""
    d = os.path.join(out_dir, "constant", "polyMesh")
    os.makedirs(d, exist_ok=True)
    npt = m.points.shape[0]
    P3 = np.concatenate([np.c_[m.points, np.zeros(npt)], np.c_[m.points, np.full(npt, m.depth)]])
    with open(os.path.join(d, "points"), "w") as f:
        f.write(_header("vectorField", "points", "constant/polyMesh"))
        f.write(f"{P3.shape[0]}\n(\n")
        f.writelines(f"({_fmt(x)} {_fmt(y)} {_fmt(z)})\n" for x, y, z in P3)
        f.write(")\n")
    fp = m.face_pts.astype(np.int64)
    side = [f"4({a} {b} {b + npt} {a + npt})" for a, b in fp]
    front, back = [], []
    for c in range(m.n_cells):
        poly = m.cell_pts[m.cell_ptr[c]:m.cell_ptr[c + 1]].astype(np.int64)
        front.append(f"{len(poly)}(" + " ".join(str(v) for v in poly[::-1]) + ")")
        back.append(f"{len(poly)}(" + " ".join(str(v + npt) for v in poly) + ")")
    faces = side + front + back
    with open(os.path.join(d, "faces"), "w") as f:
        f.write(_header("faceList", "faces", "constant/polyMesh"))
        f.write(f"{len(faces)}\n(\n" + "\n".join(faces) + "\n)\n")
    cells = np.arange(m.n_cells)
    owner = np.concatenate([m.owner.astype(np.int64), cells, cells])
    with open(os.path.join(d, "owner"), "w") as f:
        f.write(_header("labelList", "owner", "constant/polyMesh"))
        f.write(f"{owner.shape[0]}\n(\n" + "\n".join(map(str, owner)) + "\n)\n")
    with open(os.path.join(d, "neighbour"), "w") as f:
        f.write(_header("labelList", "neighbour", "constant/polyMesh"))
        f.write(f"{m.neighbour.shape[0]}\n(\n" + "\n".join(map(str, m.neighbour)) + "\n)\n")
    with open(os.path.join(d, "boundary"), "w") as f:
        f.write(_header("polyBoundaryMesh", "boundary", "constant/polyMesh"))
        f.write(f"{len(m.patches) + 1}\n(\n")
        for name, _, start, size in m.patches:
            f.write(f"    {name}\n    {{\n        type            patch;\n        nFaces          {size};\n"
                    f"        startFace       {start};\n    }}\n")
        f.write(f"    defaultFaces\n    {{\n        type            empty;\n        nFaces          {2 * m.n_cells};\n"
                f"        startFace       {m.n_faces};\n    }}\n)\n")


def _write_field(path, name, cls, dims, cells, ghosts, patches, time_name):
    vec = cls == "volVectorField"

    def vals(a):
        if vec:
            return "\n".join(f"({_fmt(x)} {_fmt(y)} 0)" for x, y in a)
        return "\n".join(_fmt(x) for x in a)

    kind = "vector" if vec else "scalar"
    with open(path, "w") as f:
        f.write(_header(cls, name, time_name))
        f.write(f"dimensions      {dims};\n\n")
        f.write(f"internalField   nonuniform List<{kind}>\n{cells.shape[0]}\n(\n{vals(cells)}\n)\n;\n\n")
        f.write("boundaryField\n{\n")
        off = 0
        for pname, _, _, size in patches:
            f.write(f"    {pname}\n    {{\n        type            calculated;\n"
                    f"        value           nonuniform List<{kind}>\n{size}\n(\n{vals(ghosts[off:off + size])}\n)\n;\n    }}\n")
            off += size
        f.write("    defaultFaces\n    {\n        type            empty;\n    }\n}\n")


def time_name(t: float) -> str:
    """OpenFOAM's time directory name (general format, 6 significant digits)."""
    return f"{t:.6g}"


def write_fields(out_dir: str, t: float, m: M.FoamMesh, FD: np.ndarray, flags: np.ndarray):
    """``<t>/p``, ``U``, ``T`` and ``shockIndicator`` like the reference's writeField
    (basicCUDAsolver.cpp:874-913): cell values and ghost values per patch; the indicator is the
    final switch type of each cell (boundary values 0)."""
    tn = time_name(t)
    d = os.path.join(out_dir, tn)
    os.makedirs(d, exist_ok=True)
    nc = m.n_cells
    cells, ghosts = FD[:nc], FD[nc:]
    _write_field(os.path.join(d, "p"), "p", "volScalarField", "[1 -1 -2 0 0 0 0]", cells[:, 0], ghosts[:, 0],
                 m.patches, tn)
    _write_field(os.path.join(d, "U"), "U", "volVectorField", "[0 1 -1 0 0 0 0]", cells[:, 1:3], ghosts[:, 1:3],
                 m.patches, tn)
    _write_field(os.path.join(d, "T"), "T", "volScalarField", "[0 0 0 1 0 0 0]", cells[:, 3], ghosts[:, 3],
                 m.patches, tn)
    si = np.asarray(flags[1:2 * nc:2], dtype=np.float64)
    _write_field(os.path.join(d, "shockIndicator"), "shockIndicator", "volScalarField", "[0 0 0 0 0 0 0]", si,
                 np.zeros(ghosts.shape[0]), m.patches, tn)
    return d


def read_field(path: str) -> np.ndarray:
    """The internal values of a field written by ``write_fields`` (nonuniform ascii lists)."""
    txt = open(path).read()
    m = re.search(r"internalField\s+nonuniform\s+List<(\w+)>\s*(\d+)\s*\((.*?)\)\s*;", txt, re.S)
    kind, n, body = m.group(1), int(m.group(2)), m.group(3)
    if kind == "vector":
        vals = np.array([[float(x) for x in s.split()] for s in re.findall(r"\(([^()]*)\)", body)])
        return vals[:n]
    return np.array([float(x) for x in body.split()])[:n]


# ----------------------------------------------------------------------------------- RBF basis files
BASIS_FILES = ("basisOwnList", "basisNeiList")


def _basis_layout(hf):
    """Per internal face and side: the stencil length (the cell itself first) and the offset of the
    face's row in the bundle's ``RBFbasis`` (2*(maxStencilSize+1) values per face, owner side then
    neighbour side)."""
    nf, maxS = hf.sizes["facesNum"], hf.sizes["maxStencilSize"]
    nb = hf.a["neighbour"].reshape(nf, 2)
    ss = hf.a["stencilSize"].astype(np.int64)
    lens = np.stack([ss[nb[:, 0]] + 1, ss[nb[:, 1]] + 1])  # (2, nf)
    base = np.arange(nf, dtype=np.int64) * 2 * (maxS + 1)
    return lens, np.stack([base, base + maxS + 1])


def write_basis_lists(system_dir: str, hf, precision: int = 17):
    """``basisOwnList`` and ``basisNeiList``: the O3 RBF weights of every internal face as OpenFOAM
    ascii ``IOList<List<scalar>>`` files, one list per face with the owner's (neighbour's) stencil
    length, the cell itself first -- the files the reference writes beside its case dictionaries
    after computing the weights (basicCUDAsolver.cpp:538-651).  The values are the double weights
    when the bundle carries them (``RBFbasis64``), else its float weights; ``precision`` significant
    digits (17 reads back bit-exact)."""
    os.makedirs(system_dir, exist_ok=True)
    w = hf.a.get("RBFbasis64")
    if w is None or w.shape[0] != hf.a["RBFbasis"].shape[0]:
        w = hf.a["RBFbasis"].astype(np.float64)
    lens, starts = _basis_layout(hf)
    fmt = f"{{:.{precision}g}}"
    for side, name in enumerate(BASIS_FILES):
        with open(os.path.join(system_dir, name), "w") as f:
            f.write(_header("scalarListList", name, "system"))
            f.write(f"{lens.shape[1]}\n(\n")
            for n, o in zip(lens[side].tolist(), starts[side].tolist()):
                f.write(f"{n}(" + " ".join(fmt.format(v) for v in w[o:o + n].tolist()) + ")\n")
            f.write(")\n")


def _read_list_list(path: str, lens: np.ndarray) -> np.ndarray:
    """The values of an ascii ``List<List<scalar>>`` whose inner lengths must equal ``lens``,
    concatenated.  Inner lists may be written on one line (``n(a b c)``) or one value per line,
    as OpenFOAM writes lists longer than ten."""
    txt = _strip_comments(open(path).read())
    m = re.search(r"FoamFile\s*\{(.*?)\}", txt, re.S)
    if m and re.search(r"format\s+binary", m.group(1)):
        raise ValueError(f"{path}: binary lists are not supported; write the case in ascii")
    body = txt[m.end():] if m else txt
    if "{" in body:
        raise ValueError(f"{path}: uniform list notation n{{v}} is not supported")
    a = np.fromstring(body.replace("(", " ").replace(")", " "), dtype=np.float64, sep=" ")
    n = lens.shape[0]
    if a.shape[0] < 1 or a[0] != n:
        raise ValueError(f"{path}: {int(a[0]) if a.shape[0] else 0} lists, the mesh has {n} internal faces")
    heads = 1 + np.concatenate([[0], np.cumsum(lens + 1)[:-1]])
    if a.shape[0] != 1 + int((lens + 1).sum()) or not np.array_equal(a[heads], lens):
        bad = np.nonzero(a[heads[heads < a.shape[0]]] != lens[heads < a.shape[0]])[0]
        face = int(bad[0]) if bad.shape[0] else int(np.searchsorted(heads, a.shape[0]))
        raise ValueError(f"{path}: the list of face {face} does not have the stencil's length "
                         f"{int(lens[min(face, n - 1)])}")
    idx = np.repeat(heads + 1, lens) + (np.arange(int(lens.sum())) - np.repeat(np.cumsum(lens) - lens, lens))
    return a[idx]


def read_basis_lists(system_dir: str, hf):
    """Replaces the bundle's O3 weights by those in ``basisOwnList``/``basisNeiList`` (the
    reference's ``recalcBasis false`` path, basicCUDAsolver.cpp:653-694): each face's double values
    go to ``RBFbasis64`` and, rounded to float, to ``RBFbasis``; entries past a stencil's length are
    zero.  The lists must match the mesh's stencils (count and length), else ValueError."""
    lens, starts = _basis_layout(hf)
    n = hf.a["RBFbasis"].shape[0]
    w64 = np.zeros(n, dtype=np.float64)
    for side, name in enumerate(BASIS_FILES):
        vals = _read_list_list(os.path.join(system_dir, name), lens[side])
        dst = np.repeat(starts[side], lens[side]) + (
            np.arange(vals.shape[0]) - np.repeat(np.cumsum(lens[side]) - lens[side], lens[side]))
        w64[dst] = vals
    hf.a["RBFbasis64"] = w64
    hf.a["RBFbasis"] = w64.astype(np.float32)
    return hf


# ----------------------------------------------------------------------------------- running a case
def run_case(case_dir: str, out_dir: str | None = None, policy: str = "mixed", device: int = 0, chunk: int = 50,
             write: bool = True):
    """The reference application's time loop on the GPU (cudaEuler2DmixO3RK3solver.cpp:38-60): read
    the case, mesh it, precompute, then step to ``endTime`` with the device CFL step (or the fixed
    ``deltaT`` when ``adjustTimeStep`` is off), landing on every write time like OpenFOAM's
    adjustableRunTime and writing ``p``, ``U``, ``T``, ``shockIndicator`` there (and the initial
    fields and ``constant/polyMesh``) under ``out_dir``.  With ``recalcBasis false`` in the case's
    fvSchemes the O3 weights come from ``system/basisOwnList``/``basisNeiList`` of ``case_dir``
    (which must exist); otherwise they are computed and, when writing, saved to
    ``out_dir/system`` (basicCUDAsolver.cpp:59,626-694).  Returns the write times, the steps taken
    and the solver's final time."""
    from .solver import CudaSolver, precompute

    case = load_case(case_dir)
    m = case.mesh
    save_basis = case.recalc_basis and write and out_dir
    hf = precompute(m, case.config, case.W, case.Wb, want_rbf64=policy == "fp64" or bool(save_basis))
    if not case.recalc_basis:
        read_basis_lists(os.path.join(case_dir, "system"), hf)
    elif save_basis:
        write_basis_lists(os.path.join(out_dir, "system"), hf)
    s = CudaSolver(hf, case.config, policy=policy, device=device)
    try:
        if write and out_dir:
            write_poly_mesh(out_dir, m)
            FD, flags = s.write_field()
            write_fields(out_dir, 0.0, m, FD, flags)
        wi = case.write_interval if case.write_interval > 0 else case.end_time
        s.set_write_interval(wi)
        dt_fixed = 0.0 if case.adjust_time_step else case.delta_t
        written = []
        k = 1
        t = 0.0
        while t < case.end_time * (1.0 - 1e-12):
            target = min(k * wi, case.end_time)
            while t < target * (1.0 - 1e-12):
                s.run(chunk, dt=dt_fixed, cfl=case.max_co, t_end=target)
                t, _, steps = s.time()
                FD, flags = s.write_field()
                if not np.isfinite(FD[:m.n_cells]).all():
                    raise FloatingPointError(f"non-finite state before t = {target}")
            if write and out_dir:
                write_fields(out_dir, target, m, FD, flags)
            written.append(target)
            k += 1
        t, _, steps = s.time()
        return {"write_times": written, "steps": steps, "time": t, "cells": m.n_cells}
    finally:
        s.close()
