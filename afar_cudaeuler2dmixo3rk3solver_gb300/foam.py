"""OpenFOAM case files for the AFAR solver: reading the dictionaries a reference case holds, a 2-D
blockMesh or a polyMesh, and writing the fields (and the mesh) back, in OpenFOAM's ascii or binary
format (controlDict ``writeFormat``).

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


# ----------------------------------------------------------------------------------- file formats
# OpenFOAM writes a file in ascii or binary (controlDict writeFormat).  The header and every
# dictionary stay text either way; in binary a list of a contiguous type (labels, scalars, vectors)
# is written as its size and then its raw bytes in parentheses, "N\n(<bytes>)" -- little-endian
# (LSB), labels of 32 or 64 bits and scalars of 64 bits as the header's arch entry says
# ("LSB;label=32;scalar=64", OpenFOAM's default build).  Files are read as bytes and decoded as
# latin-1, so text offsets are byte offsets and the raw payloads can be cut out exactly.
@dataclasses.dataclass
class _Fmt:
    binary: bool = False
    label: str = "<i4"
    scalar: str = "<f8"


def _load(path: str):
    """(raw bytes, the same as latin-1 text, the format, the offset just past the header)."""
    raw = open(path, "rb").read()
    txt = raw.decode("latin-1")
    fmt = _Fmt()
    m = re.search(r"FoamFile\s*\{([^{}]*)\}", txt)
    if not m:
        return raw, txt, fmt, 0
    head = _strip_comments(m.group(1))
    fmt.binary = re.search(r"format\s+binary", head) is not None
    arch = re.search(r'arch\s+"([^"]*)"', head)
    if arch:
        a = arch.group(1)
        if "MSB" in a:
            raise ValueError(f"{path}: big-endian (MSB) binary files are not supported")
        lab = re.search(r"label=(\d+)", a)
        sca = re.search(r"scalar=(\d+)", a)
        fmt.label = {"32": "<i4", "64": "<i8"}[lab.group(1)] if lab else "<i4"
        if sca and sca.group(1) != "64":
            raise ValueError(f"{path}: only 64-bit scalars are supported (arch {a})")
    return raw, txt, fmt, m.end()


def _binary_block(raw: bytes, txt: str, pos: int, count: int, dtype: str, path: str):
    """The payload "(<count items>)" that starts at the next "(" at or after pos: (array, end)."""
    i = pos
    while i < len(txt) and txt[i] in " \t\r\n":
        i += 1
    if count == 0 and (i >= len(txt) or txt[i] != "("):
        return np.zeros(0, dtype=dtype), i  # an empty list carries no parentheses
    if i >= len(txt) or txt[i] != "(":
        raise ValueError(f"{path}: binary list without its opening parenthesis")
    nbytes = count * np.dtype(dtype).itemsize
    end = i + 1 + nbytes
    if end >= len(raw) or txt[end] != ")":
        raise ValueError(f"{path}: binary list of {count} items is cut short")
    return np.frombuffer(raw[i + 1:end], dtype=dtype).copy(), end + 1


_SIZE = re.compile(r"\s*(\d+)")


def _binary_list(raw, txt, pos, items_dtype, per_item, path):
    """A binary "N (<bytes>)" list at pos: (array (N,) or (N, per_item), end)."""
    m = _SIZE.match(txt, pos)
    if not m:
        raise ValueError(f"{path}: binary list without its size")
    n = int(m.group(1))
    a, end = _binary_block(raw, txt, m.end(), n * per_item, items_dtype, path)
    return (a.reshape(n, per_item) if per_item > 1 else a), end


def _header(cls, obj, location=None, binary=False):
    loc = f'    location    "{location}";\n' if location is not None else ""
    arch = '    arch        "LSB;label=32;scalar=64";\n' if binary else ""
    return (f"FoamFile\n{{\n    version     2.0;\n    format      {'binary' if binary else 'ascii'};\n{arch}"
            f"    class       {cls};\n{loc}    object      {obj};\n}}\n\n")


def _binary_payload(a: np.ndarray, dtype: str) -> bytes:
    """A list's raw bytes between parentheses, as OpenFOAM writes it in binary (size excluded)."""
    return b"(" + np.ascontiguousarray(a, dtype=dtype).tobytes() + b")"


# ----------------------------------------------------------------------------------- polyMesh (2-D)
def _body(path: str) -> str:
    """A text file's content after its FoamFile header, comments removed (dictionaries: the same
    in ascii and binary files)."""
    _, txt, _, end = _load(path)
    return _strip_comments(txt[end:])


def _read_numbers(path: str, per_item: int, dtype) -> np.ndarray:
    """``N ( item ... )`` with items of ``per_item`` numbers (``(x y z)`` or a bare label): labels
    when dtype is an integer type, else scalars; ascii or binary."""
    raw, txt, fmt, end = _load(path)
    if fmt.binary:
        kind = fmt.label if np.issubdtype(np.dtype(dtype), np.integer) else fmt.scalar
        a, _ = _binary_list(raw, txt, end, kind, per_item, path)
        return a.astype(dtype)
    a = np.fromstring(_strip_comments(txt[end:]).replace("(", " ").replace(")", " "), dtype=np.float64, sep=" ")
    n = int(a[0]) if a.shape[0] else -1
    if n < 0 or a.shape[0] != 1 + n * per_item:
        raise ValueError(f"{path}: malformed list ({a.shape[0] - 1} numbers for {n} items of {per_item})")
    out = a[1:].reshape(n, per_item) if per_item > 1 else a[1:]
    return out.astype(dtype)


def _read_label_lists(path: str):
    """A ``List<labelList>`` (the polyMesh ``faces``) as CSR: offsets (N+1,), labels.  A
    ``faceCompactList`` -- how OpenFOAM writes faces in binary, and may in ascii -- is the offsets
    list followed by the labels list."""
    raw, txt, fmt, end = _load(path)
    compact = re.search(r"class\s+faceCompactList", txt[:end]) is not None
    if fmt.binary or compact:
        if fmt.binary:
            off, pos = _binary_list(raw, txt, end, fmt.label, 1, path)
            lab, _ = _binary_list(raw, txt, pos, fmt.label, 1, path)
        else:
            a = np.fromstring(_strip_comments(txt[end:]).replace("(", " ").replace(")", " "), dtype=np.float64,
                              sep=" ")
            n1 = int(a[0])
            off = a[1:1 + n1]
            lab = a[2 + n1:2 + n1 + int(a[1 + n1])]
        off, lab = off.astype(np.int64), lab.astype(np.int64)
        if off.shape[0] < 1 or off[0] != 0 or off[-1] != lab.shape[0] or np.any(np.diff(off) < 0):
            raise ValueError(f"{path}: malformed compact face list")
        return off, lab
    a = np.fromstring(_strip_comments(txt[end:]).replace("(", " -1 ").replace(")", " -2 "), dtype=np.float64, sep=" ")
    if a.shape[0] < 3 or a[1] != -1 or a[-1] != -2:
        raise ValueError(f"{path}: malformed list of lists")
    n = int(a[0])
    opens = np.nonzero(a == -1)[0][1:]
    counts = a[opens - 1].astype(np.int64)
    if opens.shape[0] != n or np.any(counts < 0) or np.any(a[opens + 1 + counts] != -2):
        raise ValueError(f"{path}: malformed list of lists ({opens.shape[0]} lists for {n})")
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    idx = np.repeat(opens + 1, counts) + (np.arange(off[-1]) - np.repeat(off[:-1], counts))
    return off, a[idx].astype(np.int64)


def _read_boundary(path: str):
    """The polyMesh ``boundary`` file: [(name, type, nFaces, startFace)] in file order."""
    out = []
    for name, body in re.findall(r'([^\s{}()";]+)\s*\{([^{}]*)\}', _body(path)):
        e = parse_foam(body)
        out.append((name, str(e.get("type", "patch")), int(e["nFaces"]), int(e["startFace"])))
    return out


def read_poly_mesh(case_dir: str, labels: dict | None = None, renumber: bool | str = False) -> M.FoamMesh:
    """The 2-D cross-section of the one-cell-deep polyMesh in ``case_dir/constant/polyMesh`` (what the
    reference's solver reads through OpenFOAM, basicCUDAsolver.cpp:122-258).

    The mesh must be extruded along z between two planes: every face with two points on each plane
    is a face of the 2-D mesh (internal, or of a boundary patch), every face on one plane lies in the
    ``empty`` patch, and each cell's face on the lower plane gives its polygon.  ``labels`` maps a
    patch's index in the boundary file (empty patches included, as fvSchemes ``CUDA { boundary {
    patch<k> ...; } }`` counts them) to its cudaEulerBCs label; a missing label is an error, like the
    reference's lookup.  Face order, owners and neighbours are kept as the file has them (the
    reference runs on the mesh as renumberMesh left it); ``renumber`` applies reverse Cuthill-McKee
    (``True``) or the Hilbert-curve order (``"hilbert"``)."""
    d = os.path.join(case_dir, "constant", "polyMesh")
    P3 = _read_numbers(os.path.join(d, "points"), 3, np.float64)
    foff, flab = _read_label_lists(os.path.join(d, "faces"))
    owner = _read_numbers(os.path.join(d, "owner"), 1, np.int64)
    neigh = _read_numbers(os.path.join(d, "neighbour"), 1, np.int64)
    bnd = _read_boundary(os.path.join(d, "boundary"))
    nF, nI = foff.shape[0] - 1, neigh.shape[0]
    if owner.shape[0] != nF or (flab.size and (flab.min() < 0 or flab.max() >= P3.shape[0])):
        raise ValueError("polyMesh: faces, owner and points do not agree")
    nc = int(max(owner.max(initial=-1), neigh.max(initial=-1))) + 1
    z = P3[:, 2]
    z0, z1 = float(z.min()), float(z.max())
    depth = z1 - z0
    tol = 1e-9 * max(depth, np.abs(P3[:, :2]).max(initial=0.0), 1e-300)
    lo, hi = np.abs(z - z0) <= tol, np.abs(z - z1) <= tol
    if depth <= 0 or not np.all(lo | hi):
        raise ValueError("polyMesh: not a one-cell-deep mesh between two planes of constant z")
    cnt = np.diff(foff)
    face_of = np.repeat(np.arange(nF), cnt)
    nlo = np.bincount(face_of, weights=lo[flab], minlength=nF).astype(np.int64)
    side = (cnt == 4) & (nlo == 2)
    front = nlo == cnt
    plane = front | (nlo == 0)
    if not np.all(side | plane):
        raise ValueError("polyMesh: a face is neither a side face nor on a z plane")
    if not np.all(side[:nI]):
        raise ValueError("polyMesh: an internal face is not a side face (not a 2-D mesh)")

    # patches: empty ones hold exactly the plane faces
    patches, keep = [], [np.arange(nI)]
    start = nI
    for k, (name, ptype, size, pstart) in enumerate(bnd):
        f = np.arange(pstart, pstart + size)
        if ptype == "empty":
            if not np.all(plane[f]):
                raise ValueError(f"polyMesh: the empty patch {name} holds side faces")
            continue
        if not np.all(side[f]):
            raise ValueError(f"polyMesh: the patch {name} holds faces on a z plane; make it empty")
        if size == 0:
            continue
        if labels is None or k not in labels:
            raise ValueError(f"no cudaEulerBCs label for patch{k} ({name}) in fvSchemes CUDA boundary")
        patches.append((name, int(labels[k]), start, size))
        keep.append(f)
        start += size
    keep = np.concatenate(keep)
    if keep.shape[0] != int(side.sum()):
        raise ValueError("polyMesh: side faces outside the internal faces and the patches")

    # 2-D points: those of the lower plane, in file order
    pid = np.full(P3.shape[0], -1, dtype=np.int64)
    pid[lo] = np.arange(int(lo.sum()))
    pts = P3[lo, :2].copy()

    # cell polygons: each cell's lower-plane face, counter-clockwise
    fr = np.nonzero(front)[0]
    cell = owner[fr]
    if fr.shape[0] != nc or np.unique(cell).shape[0] != nc:
        raise ValueError("polyMesh: every cell needs exactly one face on the lower plane")
    fr = fr[np.argsort(cell)]
    ccnt = cnt[fr]
    cptr = np.zeros(nc + 1, dtype=np.int64)
    np.cumsum(ccnt, out=cptr[1:])
    cpts = pid[flab[np.repeat(foff[fr], ccnt) + (np.arange(cptr[-1]) - np.repeat(cptr[:-1], ccnt))]]
    _, area = M._polygon_centroids(pts, cptr, cpts)
    for c in np.nonzero(area < 0)[0]:
        cpts[cptr[c]:cptr[c + 1]] = cpts[cptr[c]:cptr[c + 1]][::-1].copy()

    # 2-D faces: the lower-plane edge of each side face, ordered so (dy, -dx) points out of the owner
    sl = flab[foff[keep][:, None] + np.arange(4)[None, :]]
    on = lo[sl]
    first = np.argmax(on, axis=1)
    second = 3 - np.argmax(on[:, ::-1], axis=1)
    a, b = sl[np.arange(keep.shape[0]), first], sl[np.arange(keep.shape[0]), second]
    Q = P3[sl]  # (F, 4, 3): the face's area vector (sum of edge cross products) in x-y
    nx = np.zeros(keep.shape[0])
    ny = np.zeros(keep.shape[0])
    for i in range(4):
        p, q = Q[:, i], Q[:, (i + 1) % 4]
        nx += p[:, 1] * q[:, 2] - p[:, 2] * q[:, 1]
        ny += p[:, 2] * q[:, 0] - p[:, 0] * q[:, 2]
    pa, pb = P3[a], P3[b]
    flip = (pb[:, 1] - pa[:, 1]) * nx - (pb[:, 0] - pa[:, 0]) * ny < 0
    a, b = np.where(flip, b, a), np.where(flip, a, b)
    fpts = np.stack([pid[a], pid[b]], axis=1)
    fown = owner[keep]
    mesh = M.FoamMesh(points=pts, cell_ptr=cptr.astype(np.int32), cell_pts=cpts.astype(np.int32),
                      face_pts=fpts.astype(np.int32), owner=fown.astype(np.int32),
                      neighbour=neigh.astype(np.int32), patches=patches, depth=depth)
    return M.renumber_mesh(mesh, "rcm" if renumber is True else renumber) if renumber else mesh


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


_NONUNIFORM = re.compile(r"nonuniform\s+List<(scalar|vector)>\s*(\d+)\s*\(")
_VECTOR_BODY = re.compile(r"(?:\s*\([^()]*\))*\s*\)")
_SLIP = ("slip", "symmetryPlane", "symmetry")


def read_field_dict(path: str):
    """A volField file as a FoamDict, its ``nonuniform List<...>`` values read by numpy into arrays
    ((N,) for scalars, (N, 3) for vectors) instead of being tokenised; ascii or binary."""
    raw, txt, fmt, hend = _load(path)
    if fmt.binary:
        return _read_binary_field_dict(raw, txt, fmt, hend, path)
    txt = _strip_comments(txt)
    arrays, parts, i = [], [], 0
    while True:
        m = _NONUNIFORM.search(txt, i)
        if not m:
            break
        kind, n = m.group(1), int(m.group(2))
        if kind == "scalar":
            end = txt.index(")", m.end()) + 1
        else:
            e = _VECTOR_BODY.match(txt, m.end())
            if not e:
                raise ValueError(f"{path}: malformed vector list")
            end = e.end()
        a = np.fromstring(txt[m.end():end - 1].replace("(", " ").replace(")", " "), dtype=np.float64, sep=" ")
        k = 3 if kind == "vector" else 1
        if a.shape[0] != n * k:
            raise ValueError(f"{path}: a list of {n} {kind}s holds {a.shape[0]} numbers")
        arrays.append(a.reshape(n, 3) if k == 3 else a)
        parts += [txt[i:m.start()], f" __afar_list_{len(arrays) - 1}__ "]
        i = end
    parts.append(txt[i:])
    return _resolve_lists(parse_foam("".join(parts)), arrays)


_NONUNIFORM_BIN = re.compile(r"nonuniform\s+List<(scalar|vector)>\s*(\d+)")


def _resolve_lists(d, arrays):
    def resolve(v):
        if isinstance(v, str) and v.startswith("__afar_list_"):
            return arrays[int(v[12:-2])]
        if isinstance(v, list):
            return [resolve(x) for x in v]
        if isinstance(v, dict):
            for key in v:
                v[key] = resolve(v[key])
        return v

    return resolve(d)


def _read_binary_field_dict(raw, txt, fmt, hend, path):
    """read_field_dict of a binary file: each nonuniform list's payload is cut out of the bytes and
    the text around the payloads parsed as a dictionary."""
    arrays, parts, i = [], [], hend
    while True:
        m = _NONUNIFORM_BIN.search(txt, i)
        if not m:
            break
        k = 3 if m.group(1) == "vector" else 1
        a, end = _binary_block(raw, txt, m.end(), int(m.group(2)) * k, fmt.scalar, path)
        arrays.append(a.reshape(-1, 3) if k == 3 else a)
        parts += [txt[i:m.start()], f" __afar_list_{len(arrays) - 1}__ "]
        i = end
    parts.append(txt[i:])
    return _resolve_lists(parse_foam(_strip_comments("".join(parts))), arrays)


def _values(v, n, is_vector, what):
    """An entry's value as (n, 2) velocities (x, y) or (n, 1) scalars."""
    if isinstance(v, list) and len(v) == 2 and v[0] == "uniform":
        a = np.asarray(v[1], dtype=np.float64)
        return np.tile(a[:2] if is_vector else np.array([float(a)]), (n, 1))
    if isinstance(v, np.ndarray):
        if v.shape[0] != n:
            raise ValueError(f"{what}: {v.shape[0]} values for {n}")
        return v[:, :2].copy() if is_vector else v[:, None].copy()
    raise ValueError(f"{what}: expected uniform or nonuniform values, got {v!r}")


def _field_values(fdict, m: M.FoamMesh, is_vector):
    """Cell values and the initial ghost value of every boundary face, the patch values OpenFOAM
    gives the reference at construction (basicCUDAsolver.cpp:161-192): ``value`` where the patch
    type stores one, the owner cell's value for zeroGradient and other value-less types, the
    owner's tangential velocity for slip/symmetry (scalars: the owner's value), zero velocity for
    noSlip."""
    nc = m.n_cells
    cells = _values(fdict["internalField"], nc, is_vector, "internalField")
    bf = fdict.get("boundaryField", {})
    out = []
    for name, _, start, size in m.patches:
        spec = bf.get(name, {})
        ptype = str(spec.get("type", "zeroGradient"))
        own = m.owner[start:start + size]
        if ptype in _SLIP and is_vector:
            pa, pb = m.points[m.face_pts[start:start + size, 0]], m.points[m.face_pts[start:start + size, 1]]
            nrm = np.stack([pb[:, 1] - pa[:, 1], pa[:, 0] - pb[:, 0]], axis=1)
            nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
            u = cells[own]
            out.append(u - nrm * np.sum(u * nrm, axis=1, keepdims=True))
        elif ptype == "noSlip" and is_vector:
            out.append(np.zeros((size, 2)))
        elif "value" in spec and ptype not in ("zeroGradient",) + _SLIP:
            out.append(_values(spec["value"], size, is_vector, f"{name} value"))
        else:
            out.append(cells[own])
    ghosts = np.concatenate(out) if out else np.zeros((0, cells.shape[1]))
    return cells, ghosts


def load_case(case_dir: str, renumber: bool = True) -> FoamCase:
    """The reference case in ``case_dir`` as solver inputs: the meshed cross-section, the case
    configuration (fvSchemes ``CUDA`` and ``gaussQuadrature``, controlDict ``maxCo``), the initial
    cell states and ghost states, and the time controls.  The mesh is ``constant/polyMesh`` when the
    case has one (as the reference reads it), else ``system/blockMeshDict`` meshed here and, with
    ``renumber``, reverse Cuthill-McKee ordered (the blockMesh + renumberMesh steps).  Initial
    fields may be uniform or nonuniform."""
    from .solver import CaseConfig

    sysd = os.path.join(case_dir, "system")
    schemes = read_foam(os.path.join(sysd, "fvSchemes"))
    control = read_foam(os.path.join(sysd, "controlDict"))
    cuda = schemes["CUDA"]
    gq = schemes.get("gaussQuadrature", {})
    blabels = cuda.get("boundary", {})
    if os.path.exists(os.path.join(case_dir, "constant", "polyMesh", "faces")):
        by_index = {int(k[5:]): int(v) for k, v in blabels.items() if re.fullmatch(r"patch\d+", str(k))}
        m = read_poly_mesh(case_dir, by_index)
    else:
        bmd = read_foam(os.path.join(sysd, "blockMeshDict"))
        bnd = bmd.get("boundary", [])
        names = [bnd[k] for k in range(0, len(bnd), 2)]
        labels = {name: int(blabels[f"patch{k}"]) for k, name in enumerate(names) if f"patch{k}" in blabels}
        m = block_mesh_2d(bmd, labels, renumber=renumber)
    max_co = float(control.get("maxCo", 0.5))
    cfg = CaseConfig(R=float(cuda["R"]), Cv=float(cuda["Cv"]), CFL=max_co,
                     stencilType=str(cuda.get("stencilType", "edgeNeighbour")),
                     shapeFactor=float(schemes.get("shapeFactor", 10.0)),
                     cOrder=int(gq.get("cOrder", 5)), fOrder=int(gq.get("fOrder", 4)))
    zero = os.path.join(case_dir, "0")
    p, pb = _field_values(read_field_dict(os.path.join(zero, "p")), m, False)
    U, Ub = _field_values(read_field_dict(os.path.join(zero, "U")), m, True)
    T, Tb = _field_values(read_field_dict(os.path.join(zero, "T")), m, False)
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
def _fmt(v):
    return f"{v:.9g}"


def write_poly_mesh(out_dir: str, m: M.FoamMesh, binary: bool = False):
    """``constant/polyMesh`` of the one-cell-deep 3-D mesh: points on z = 0 and z = depth, a quad
    per 2-D face (internal faces first, then the named patches), and the front and back polygons
    of every cell in the empty patch ``defaultFaces``; in ascii, or in OpenFOAM's binary form
    (faces as a ``faceCompactList``)."""
    d = os.path.join(out_dir, "constant", "polyMesh")
    os.makedirs(d, exist_ok=True)
    npt = m.points.shape[0]
    P3 = np.concatenate([np.c_[m.points, np.zeros(npt)], np.c_[m.points, np.full(npt, m.depth)]])
    if binary:
        return _write_poly_mesh_binary(d, m, P3)
    with open(os.path.join(d, "points"), "w") as f:
        f.write(_header("vectorField", "points", "constant/polyMesh"))
        f.write(f"{P3.shape[0]}\n(\n")
        f.writelines(f"({x!r} {y!r} {z!r})\n" for x, y, z in P3.tolist())  # shortest exact form
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
    _write_boundary(d, m, False)


def _poly_faces(m: M.FoamMesh):
    """The 3-D faces as CSR (offsets, labels): side quads, then front and back cell polygons."""
    npt = m.points.shape[0]
    fp = m.face_pts.astype(np.int64)
    side = np.stack([fp[:, 0], fp[:, 1], fp[:, 1] + npt, fp[:, 0] + npt], axis=1).reshape(-1)
    cnt = np.diff(m.cell_ptr.astype(np.int64))
    polys = m.cell_pts.astype(np.int64)
    # each cell's polygon reversed (front, normal -z) and as it is, on the upper plane (back)
    rev = np.concatenate([polys[m.cell_ptr[c]:m.cell_ptr[c + 1]][::-1] for c in range(m.n_cells)]) \
        if m.n_cells else np.zeros(0, dtype=np.int64)
    labels = np.concatenate([side, rev, polys + npt])
    counts = np.concatenate([np.full(fp.shape[0], 4), cnt, cnt])
    off = np.zeros(counts.shape[0] + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    return off, labels


def _write_poly_mesh_binary(d, m, P3):
    cells = np.arange(m.n_cells)
    owner = np.concatenate([m.owner.astype(np.int64), cells, cells])
    off, lab = _poly_faces(m)
    for name, cls, parts in (
            ("points", "vectorField", [(P3.shape[0], P3, "<f8")]),
            ("faces", "faceCompactList", [(off.shape[0], off, "<i4"), (lab.shape[0], lab, "<i4")]),
            ("owner", "labelList", [(owner.shape[0], owner, "<i4")]),
            ("neighbour", "labelList", [(m.neighbour.shape[0], m.neighbour, "<i4")])):
        with open(os.path.join(d, name), "wb") as f:
            f.write(_header(cls, name, "constant/polyMesh", binary=True).encode())
            for n, a, dt in parts:
                f.write(f"\n{n}\n".encode() + _binary_payload(a, dt) + b"\n")
            f.write(b"\n")
    _write_boundary(d, m, True)


def _write_boundary(d, m, binary):
    with open(os.path.join(d, "boundary"), "w") as f:
        f.write(_header("polyBoundaryMesh", "boundary", "constant/polyMesh", binary=binary))
        f.write(f"{len(m.patches) + 1}\n(\n")
        for name, _, start, size in m.patches:
            f.write(f"    {name}\n    {{\n        type            patch;\n        nFaces          {size};\n"
                    f"        startFace       {start};\n    }}\n")
        f.write(f"    defaultFaces\n    {{\n        type            empty;\n        nFaces          {2 * m.n_cells};\n"
                f"        startFace       {m.n_faces};\n    }}\n)\n")


def _write_field(path, name, cls, dims, cells, ghosts, patches, time_name, binary=False):
    vec = cls == "volVectorField"
    if binary:
        return _write_field_binary(path, name, cls, dims, cells, ghosts, patches, time_name, vec)

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


def _write_field_binary(path, name, cls, dims, cells, ghosts, patches, time_name, vec):
    """The field in OpenFOAM's binary form: the dictionary as text, each nonuniform list as its size
    and raw 64-bit values (vectors with a zero z component, double precision, so no rounding)."""
    kind = "vector" if vec else "scalar"

    def block(a):
        a = np.asarray(a, dtype=np.float64)
        if vec:
            a = np.c_[a, np.zeros(a.shape[0])]
        return f"nonuniform List<{kind}> \n{a.shape[0]}\n".encode() + _binary_payload(a, "<f8")

    with open(path, "wb") as f:
        f.write(_header(cls, name, time_name, binary=True).encode())
        f.write(f"dimensions      {dims};\n\ninternalField   ".encode() + block(cells) + b";\n\nboundaryField\n{\n")
        off = 0
        for pname, _, _, size in patches:
            f.write(f"    {pname}\n    {{\n        type            calculated;\n        value           ".encode()
                    + block(ghosts[off:off + size]) + b";\n    }\n")
            off += size
        f.write(b"    defaultFaces\n    {\n        type            empty;\n    }\n}\n")


def time_name(t: float) -> str:
    """OpenFOAM's time directory name (general format, 6 significant digits)."""
    return f"{t:.6g}"


def write_fields(out_dir: str, t: float, m: M.FoamMesh, FD: np.ndarray, flags: np.ndarray, binary: bool = False):
    """``<t>/p``, ``U``, ``T`` and ``shockIndicator`` like the reference's writeField
    (basicCUDAsolver.cpp:874-913): cell values and ghost values per patch; the indicator is the
    final switch type of each cell (boundary values 0).  ascii (9 significant digits) or binary
    (the doubles themselves)."""
    tn = time_name(t)
    d = os.path.join(out_dir, tn)
    os.makedirs(d, exist_ok=True)
    nc = m.n_cells
    cells, ghosts = FD[:nc], FD[nc:]
    _write_field(os.path.join(d, "p"), "p", "volScalarField", "[1 -1 -2 0 0 0 0]", cells[:, 0], ghosts[:, 0],
                 m.patches, tn, binary)
    _write_field(os.path.join(d, "U"), "U", "volVectorField", "[0 1 -1 0 0 0 0]", cells[:, 1:3], ghosts[:, 1:3],
                 m.patches, tn, binary)
    _write_field(os.path.join(d, "T"), "T", "volScalarField", "[0 0 0 1 0 0 0]", cells[:, 3], ghosts[:, 3],
                 m.patches, tn, binary)
    si = np.asarray(flags[1:2 * nc:2], dtype=np.float64)
    _write_field(os.path.join(d, "shockIndicator"), "shockIndicator", "volScalarField", "[0 0 0 0 0 0 0]", si,
                 np.zeros(ghosts.shape[0]), m.patches, tn, binary)
    return d


def read_field(path: str) -> np.ndarray:
    """The internal values of a field file with a nonuniform internalField, ascii or binary:
    (N,) scalars or (N, 3) vectors."""
    v = read_field_dict(path)["internalField"]
    if isinstance(v, list) and len(v) == 2 and v[0] == "nonuniform":  # a short ascii list kept as tokens
        v = np.asarray(v[1], dtype=np.float64)
    return np.asarray(v, dtype=np.float64)


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


def write_basis_lists(system_dir: str, hf, precision: int = 17, binary: bool = False):
    """``basisOwnList`` and ``basisNeiList``: the O3 RBF weights of every internal face as OpenFOAM
    ascii ``IOList<List<scalar>>`` files, one list per face with the owner's (neighbour's) stencil
    length, the cell itself first -- the files the reference writes beside its case dictionaries
    after computing the weights (basicCUDAsolver.cpp:538-651).  The values are the double weights
    when the bundle carries them (``RBFbasis64``), else its float weights; ``precision`` significant
    digits (17 reads back bit-exact).  In binary each face's list is its length and its raw doubles,
    inside the outer list's text parentheses, as OpenFOAM writes a list of lists."""
    os.makedirs(system_dir, exist_ok=True)
    w = hf.a.get("RBFbasis64")
    if w is None or w.shape[0] != hf.a["RBFbasis"].shape[0]:
        w = hf.a["RBFbasis"].astype(np.float64)
    lens, starts = _basis_layout(hf)
    fmt = f"{{:.{precision}g}}"
    for side, name in enumerate(BASIS_FILES):
        if binary:
            with open(os.path.join(system_dir, name), "wb") as f:
                f.write(_header("scalarListList", name, "system", binary=True).encode())
                f.write(f"\n{lens.shape[1]}\n(\n".encode())
                for n, o in zip(lens[side].tolist(), starts[side].tolist()):
                    f.write(f"\n{n}\n".encode() + _binary_payload(w[o:o + n], "<f8") + b"\n")
                f.write(b")\n")
            continue
        with open(os.path.join(system_dir, name), "w") as f:
            f.write(_header("scalarListList", name, "system"))
            f.write(f"{lens.shape[1]}\n(\n")
            for n, o in zip(lens[side].tolist(), starts[side].tolist()):
                f.write(f"{n}(" + " ".join(fmt.format(v) for v in w[o:o + n].tolist()) + ")\n")
            f.write(")\n")


def _read_list_list(path: str, lens: np.ndarray) -> np.ndarray:
    """The values of an ascii ``List<List<scalar>>`` whose inner lengths must equal ``lens``,
    concatenated.  Inner lists may be written on one line (``n(a b c)``) or one value per line,
    as OpenFOAM writes lists longer than ten; in a binary file each inner list is its length and
    raw doubles."""
    raw, txt, fmt, hend = _load(path)
    if fmt.binary:
        return _read_binary_list_list(raw, txt, fmt, hend, lens, path)
    body = _strip_comments(txt[hend:])
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


def _read_binary_list_list(raw, txt, fmt, pos, lens, path):
    m = _SIZE.match(txt, pos)
    n = lens.shape[0]
    if not m or int(m.group(1)) != n:
        raise ValueError(f"{path}: {int(m.group(1)) if m else 0} lists, the mesh has {n} internal faces")
    i = m.end()
    while txt[i] in " \t\r\n":
        i += 1
    if txt[i] != "(":
        raise ValueError(f"{path}: list of lists without its opening parenthesis")
    i += 1
    out = []
    for face in range(n):
        a, i = _binary_list(raw, txt, i, fmt.scalar, 1, path)
        if a.shape[0] != lens[face]:
            raise ValueError(f"{path}: the list of face {face} does not have the stencil's length {int(lens[face])}")
        out.append(a)
    return np.concatenate(out) if out else np.zeros(0)


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
    binary = str(read_foam(os.path.join(case_dir, "system", "controlDict")).get("writeFormat", "ascii")) == "binary"
    m = case.mesh
    save_basis = case.recalc_basis and write and out_dir
    hf = precompute(m, case.config, case.W, case.Wb, want_rbf64=policy == "fp64" or bool(save_basis))
    if not case.recalc_basis:
        read_basis_lists(os.path.join(case_dir, "system"), hf)
    elif save_basis:
        write_basis_lists(os.path.join(out_dir, "system"), hf, binary=binary)
    s = CudaSolver(hf, case.config, policy=policy, device=device)
    try:
        if write and out_dir:
            write_poly_mesh(out_dir, m, binary=binary)
            FD, flags = s.write_field()
            write_fields(out_dir, 0.0, m, FD, flags, binary=binary)
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
                write_fields(out_dir, target, m, FD, flags, binary=binary)
            written.append(target)
            k += 1
        t, _, steps = s.time()
        return {"write_times": written, "steps": steps, "time": t, "cells": m.n_cells}
    finally:
        s.close()
