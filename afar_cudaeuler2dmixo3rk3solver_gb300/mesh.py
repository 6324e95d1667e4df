"""Synthetic 2-D meshes in OpenFOAM polyMesh form, plus the initial fields of the workloads.

The reference solver reads an OpenFOAM case (``blockMesh`` + ``renumberMesh``): points, faces,
owner, neighbour and boundary patches of a one-cell-deep 3-D mesh (reference
``src/CUDA/cudaEuler2DmixO3RK3/basicCUDAsolver.cpp:122-258``, ``README.md:65-77``).  This module
builds the same arrays for the 2-D cross-section directly:

* ``points``      (Np, 2) float64  vertex coordinates (x, y)
* ``cell_ptr``    (Nc+1,) int32    CSR offsets into ``cell_pts``
* ``cell_pts``    (sum,)  int32    polygon vertices of each cell, counter-clockwise
* ``face_pts``    (NF, 2) int32    the two vertices of each face (an edge of the cross-section),
                                   ordered so that the face normal points out of the owner
* ``owner``       (NF,)   int32    owner cell of every face
* ``neighbour``   (Nf,)   int32    neighbour cell of every internal face (owner < neighbour)
* ``patches``     list of (name, label, start, size): boundary faces are stored patch by patch
                                   after the ``Nf`` internal faces; ``label`` is the cudaEulerBCs
                                   patch label of the reference (``src/CUDA/BCs/2D/cudaEulerBCs.h:45-62``)

Internal faces follow OpenFOAM's upper-triangular order (sorted by owner, then neighbour) and the
cells are renumbered by reverse Cuthill-McKee, the job ``renumberMesh`` does for the reference.
Everything here is workload generation; the solver path itself is native code.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# cudaEulerBCs patch labels (reference src/CUDA/BCs/2D/cudaEulerBCs.h:56-61)
BC_CONST_T_WALL = 0
BC_ADIABATIC_WALL = 1
BC_SLIP = 2
BC_FIXED_VALUE = 3
BC_OUTLET = 4
BC_FIXED_VALUE2 = 5
BC_FIXED_INITIAL = 6  # the ghost keeps the state given for it at set-up (an inflow of any value)


@dataclasses.dataclass
class FoamMesh:
    points: np.ndarray
    cell_ptr: np.ndarray
    cell_pts: np.ndarray
    face_pts: np.ndarray
    owner: np.ndarray
    neighbour: np.ndarray
    patches: list  # [(name, label, start, size)]
    depth: float = 1.0
    period: tuple = (0.0, 0.0)  # periodic mesh: (Lx, Ly), 0 = not periodic in that direction
    point_alias: np.ndarray | None = None  # periodic mesh: representative of each point's images

    @property
    def n_cells(self) -> int:
        return int(self.cell_ptr.shape[0] - 1)

    @property
    def n_internal_faces(self) -> int:
        return int(self.neighbour.shape[0])

    @property
    def n_faces(self) -> int:
        return int(self.owner.shape[0])

    @property
    def n_boundary_faces(self) -> int:
        return self.n_faces - self.n_internal_faces

    # ---------------------------------------------------------------- geometry (for tests/inits)
    def cell_centres(self) -> np.ndarray:
        """Area centroids of the cell polygons (what OpenFOAM's ``mesh.C()`` gives in 2-D)."""
        xy, area = _polygon_centroids(self.points, self.cell_ptr, self.cell_pts)
        return xy

    def cell_areas(self) -> np.ndarray:
        _, area = _polygon_centroids(self.points, self.cell_ptr, self.cell_pts)
        return area

    def face_centres(self) -> np.ndarray:
        p = self.points
        return 0.5 * (p[self.face_pts[:, 0]] + p[self.face_pts[:, 1]])

    def boundary_face_centres(self) -> np.ndarray:
        return self.face_centres()[self.n_internal_faces:]


def _polygon_centroids(points, cell_ptr, cell_pts):
    nv = np.diff(cell_ptr)
    idx = np.arange(cell_pts.shape[0])
    nxt = idx + 1
    nxt[cell_ptr[1:] - 1] = cell_ptr[:-1]
    a = points[cell_pts]
    b = points[cell_pts[nxt]]
    cross = a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]
    cell_of = np.repeat(np.arange(nv.shape[0]), nv)
    area2 = np.bincount(cell_of, weights=cross, minlength=nv.shape[0])
    cx = np.bincount(cell_of, weights=(a[:, 0] + b[:, 0]) * cross, minlength=nv.shape[0])
    cy = np.bincount(cell_of, weights=(a[:, 1] + b[:, 1]) * cross, minlength=nv.shape[0])
    area = 0.5 * area2
    return np.stack([cx / (3.0 * area2), cy / (3.0 * area2)], axis=1), area


def _rcm_permutation(n_cells, own, nei):
    """Reverse Cuthill-McKee order of the cell graph (scipy), the renumberMesh step."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee

    rows = np.concatenate([own, nei])
    cols = np.concatenate([nei, own])
    g = sp.csr_matrix((np.ones(rows.shape[0], dtype=np.int8), (rows, cols)), shape=(n_cells, n_cells))
    return np.asarray(reverse_cuthill_mckee(g, symmetric_mode=True), dtype=np.int64)


def _hilbert_permutation(xy, bits=16):
    """Cells sorted along a Hilbert curve through their centres (new -> old).  Consecutive cells
    then form compact patches, so the stencils of a 128-cell tile share most of their members
    (reverse Cuthill-McKee makes a tile a thin strip along its front instead).  The curve index is
    the classic quadrant-rotation walk from the coarsest level down (Hilbert 1891; the
    ``xy2d`` form of Butz's algorithm), on a 2^bits grid over the bounding square."""
    n = 1 << bits
    xy = np.asarray(xy, dtype=np.float64)
    if xy.shape[0] == 0:
        return np.zeros(0, dtype=np.int64)
    lo = xy.min(axis=0)
    span = float((xy.max(axis=0) - lo).max()) or 1.0
    q = np.minimum(((xy - lo) * (n / span)).astype(np.int64), n - 1)
    x, y = q[:, 0].copy(), q[:, 1].copy()
    d = np.zeros(xy.shape[0], dtype=np.int64)
    s = n >> 1
    while s > 0:
        rx = ((x & s) > 0).astype(np.int64)
        ry = ((y & s) > 0).astype(np.int64)
        d += s * s * ((3 * rx) ^ ry)
        # turn the quadrant so its sub-curve runs like the parent's: reflect, then transpose
        refl = (ry == 0) & (rx == 1)
        x = np.where(refl, n - 1 - x, x)
        y = np.where(refl, n - 1 - y, y)
        swap = ry == 0
        x, y = np.where(swap, y, x), np.where(swap, x, y)
        s >>= 1
    return np.argsort(d, kind="stable").astype(np.int64)


def _cell_permutation(renumber, nc, own, nei, centres):
    """new -> old cell order: reverse Cuthill-McKee (``True`` or "rcm"), a Hilbert curve through
    the cell centres ("hilbert"), or the given order (``False``)."""
    if renumber == "hilbert":
        return _hilbert_permutation(centres())
    if renumber is True or renumber == "rcm":
        return _rcm_permutation(nc, own, nei)
    if renumber is False or renumber is None:
        return np.arange(nc, dtype=np.int64)
    raise ValueError(f"unknown cell order {renumber!r}: True/'rcm', 'hilbert' or False")


def build_foam_mesh(points, cell_ptr, cell_pts, classify, patch_defs, renumber=True, depth=1.0, alias=None,
                    period=(0.0, 0.0)):
    """Assemble OpenFOAM-ordered face lists from cell polygons.

    ``classify(xm, ym) -> patch index`` assigns each boundary edge (by its midpoint) to one of
    ``patch_defs = [(name, label), ...]``.  Polygons must be counter-clockwise.  ``alias`` (periodic
    meshes) maps every point to one representative of its periodic images: edges are matched on
    representatives, so the two sides of a period meet in internal faces whose points (and so
    coordinates) are the owner's.
    """
    points = np.ascontiguousarray(points, dtype=np.float64)
    cell_ptr = np.ascontiguousarray(cell_ptr, dtype=np.int64)
    cell_pts = np.ascontiguousarray(cell_pts, dtype=np.int64)
    nc = cell_ptr.shape[0] - 1
    nv = np.diff(cell_ptr)
    cell_of = np.repeat(np.arange(nc, dtype=np.int64), nv)
    idx = np.arange(cell_pts.shape[0])
    nxt = idx + 1
    nxt[cell_ptr[1:] - 1] = cell_ptr[:-1]
    a = cell_pts
    b = cell_pts[nxt]
    ka, kb = (a, b) if alias is None else (np.asarray(alias)[a], np.asarray(alias)[b])
    lo = np.minimum(ka, kb)
    hi = np.maximum(ka, kb)
    key = lo * points.shape[0] + hi
    order = np.argsort(key, kind="stable")
    ks = key[order]
    same_next = np.zeros(ks.shape[0], dtype=bool)
    same_next[:-1] = ks[1:] == ks[:-1]
    if np.any(same_next[:-1] & same_next[1:]):
        raise ValueError("non-manifold mesh: an edge is shared by more than two cells")
    first = np.nonzero(same_next)[0]
    he_i = order[first]
    he_j = order[first + 1]
    paired = np.zeros(ks.shape[0], dtype=bool)
    paired[first] = True
    paired[first + 1] = True
    single = order[~paired]

    ci = cell_of[he_i]
    cj = cell_of[he_j]
    perm = _cell_permutation(renumber, nc, ci, cj,
                             lambda: _polygon_centroids(points, cell_ptr, cell_pts)[0])  # new -> old
    inv = np.empty(nc, dtype=np.int64)
    inv[perm] = np.arange(nc)
    ni = inv[ci]
    nj = inv[cj]
    own = np.minimum(ni, nj)
    nei = np.maximum(ni, nj)
    # half-edge as traversed by the owner keeps the normal pointing owner -> neighbour
    own_he = np.where(ni < nj, he_i, he_j)
    fo = np.lexsort((nei, own))
    own = own[fo]
    nei = nei[fo]
    own_he = own_he[fo]
    face_pts_int = np.stack([a[own_he], b[own_he]], axis=1)

    # boundary faces, grouped by patch, then by owner
    bown = inv[cell_of[single]]
    ba = a[single]
    bb = b[single]
    xm = 0.5 * (points[ba, 0] + points[bb, 0])
    ym = 0.5 * (points[ba, 1] + points[bb, 1])
    pidx = np.asarray(classify(xm, ym), dtype=np.int64) if xm.size else np.zeros(0, dtype=np.int64)
    bo = np.lexsort((bown, pidx))
    bown = bown[bo]
    pidx = pidx[bo]
    face_pts_b = np.stack([ba[bo], bb[bo]], axis=1)

    nf = own.shape[0]
    patches = []
    start = nf
    for p, (name, label) in enumerate(patch_defs):
        size = int(np.count_nonzero(pidx == p))
        patches.append((name, int(label), start, size))
        start += size

    # renumbered cell polygons
    new_nv = nv[perm]
    new_ptr = np.zeros(nc + 1, dtype=np.int64)
    np.cumsum(new_nv, out=new_ptr[1:])
    gather = (cell_ptr[perm][:, None] + np.arange(new_nv.max())[None, :])
    mask = np.arange(new_nv.max())[None, :] < new_nv[:, None]
    new_pts = cell_pts[gather[mask]]

    return FoamMesh(
        points=points,
        cell_ptr=new_ptr.astype(np.int32),
        cell_pts=new_pts.astype(np.int32),
        face_pts=np.concatenate([face_pts_int, face_pts_b]).astype(np.int32),
        owner=np.concatenate([own, bown]).astype(np.int32),
        neighbour=nei.astype(np.int32),
        patches=patches,
        depth=float(depth),
        period=tuple(float(v) for v in period),
        point_alias=None if alias is None else np.ascontiguousarray(alias, dtype=np.int32),
    )


def renumber_mesh(m: FoamMesh, order="rcm") -> FoamMesh:
    """``m`` with its cells in reverse Cuthill-McKee order (renumberMesh; ``order="hilbert"``: along
    a Hilbert curve through the cell centres): internal faces back in upper-triangular order (a
    face whose owner and neighbour swap has its points swapped, so its normal still leaves the
    owner), boundary faces sorted by owner within each patch."""
    nc, nf = m.n_cells, m.n_internal_faces
    own = m.owner.astype(np.int64)
    nei = m.neighbour.astype(np.int64)
    perm = _cell_permutation(order, nc, own[:nf], nei,
                             lambda: _polygon_centroids(m.points, m.cell_ptr, m.cell_pts)[0])
    inv = np.empty(nc, dtype=np.int64)
    inv[perm] = np.arange(nc)
    o, n = inv[own[:nf]], inv[nei]
    swap = o > n
    fp = m.face_pts.astype(np.int64).copy()
    fp[:nf][swap] = fp[:nf][swap][:, ::-1]
    o, n = np.minimum(o, n), np.maximum(o, n)
    fo = np.lexsort((n, o))
    bown = inv[own[nf:]]
    border = []
    for _, _, start, size in m.patches:
        seg = np.arange(start - nf, start - nf + size)
        border.append(seg[np.argsort(bown[seg], kind="stable")])
    bo = np.concatenate(border) if border else np.zeros(0, dtype=np.int64)
    nv = np.diff(m.cell_ptr.astype(np.int64))[perm]
    ptr = np.zeros(nc + 1, dtype=np.int64)
    np.cumsum(nv, out=ptr[1:])
    old = m.cell_ptr.astype(np.int64)[perm]
    pts = m.cell_pts[np.repeat(old, nv) + (np.arange(ptr[-1]) - np.repeat(ptr[:-1], nv))]
    return dataclasses.replace(
        m, cell_ptr=ptr.astype(np.int32), cell_pts=pts.astype(np.int32),
        face_pts=np.concatenate([fp[:nf][fo], fp[nf:][bo]]).astype(np.int32),
        owner=np.concatenate([o[fo], bown[bo]]).astype(np.int32), neighbour=n[fo].astype(np.int32))


# ------------------------------------------------------------------------------------ generators
def quad_grid(nx, ny, x0=0.0, x1=1.0, y0=0.0, y1=1.0, classify=None, patch_defs=None,
              renumber=True, jitter=0.0, seed=0, tri_mask=None):
    """Structured quad grid; cells where ``tri_mask(xc, yc)`` is true are split into two triangles
    (seeded diagonal), which gives a conforming mixed quad/triangle mesh."""
    xs = np.linspace(x0, x1, nx + 1)
    ys = np.linspace(y0, y1, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel()], axis=1)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        hx = (x1 - x0) / nx
        hy = (y1 - y0) / ny
        inner = (X.ravel() > x0) & (X.ravel() < x1) & (Y.ravel() > y0) & (Y.ravel() < y1)
        d = rng.uniform(-jitter, jitter, size=(pts.shape[0], 2)) * np.array([hx, hy])
        pts[inner] += d[inner]
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    I = I.ravel()
    J = J.ravel()
    v00 = I * (ny + 1) + J
    v10 = (I + 1) * (ny + 1) + J
    v11 = (I + 1) * (ny + 1) + J + 1
    v01 = I * (ny + 1) + J + 1
    quads = np.stack([v00, v10, v11, v01], axis=1)
    if tri_mask is None:
        cell_ptr = np.arange(0, 4 * quads.shape[0] + 1, 4)
        cell_pts = quads.ravel()
    else:
        xc = pts[quads, 0].mean(axis=1)
        yc = pts[quads, 1].mean(axis=1)
        split = np.asarray(tri_mask(xc, yc), dtype=bool)
        rng = np.random.default_rng(seed + 1)
        diag = rng.integers(0, 2, size=quads.shape[0]).astype(bool)
        q = quads[~split]
        s = quads[split]
        d = diag[split]
        t1 = np.where(d[:, None], s[:, [0, 1, 2]], s[:, [0, 1, 3]])
        t2 = np.where(d[:, None], s[:, [0, 2, 3]], s[:, [1, 2, 3]])
        # cell order: keep spatial locality by interleaving through the original grid order
        ids_q = np.nonzero(~split)[0]
        ids_s = np.nonzero(split)[0]
        polys = [None] * 0
        nq = q.shape[0]
        nt = 2 * s.shape[0]
        keys = np.concatenate([ids_q * 2.0, ids_s * 2.0, ids_s * 2.0 + 1.0])
        sizes = np.concatenate([np.full(nq, 4), np.full(nt, 3)])
        flat = [q, t1, t2]
        order = np.argsort(keys, kind="stable")
        sizes = sizes[order]
        cell_ptr = np.zeros(sizes.shape[0] + 1, dtype=np.int64)
        np.cumsum(sizes, out=cell_ptr[1:])
        allv = np.full((nq + nt, 4), -1, dtype=np.int64)
        allv[:nq] = q
        allv[nq:nq + s.shape[0], :3] = t1
        allv[nq + s.shape[0]:, :3] = t2
        allv = allv[order]
        cell_pts = allv[allv >= 0]
        del polys, flat
    if classify is None:
        eps = 1e-12 * max(x1 - x0, y1 - y0)

        def classify(xm, ym):
            out = np.zeros(xm.shape[0], dtype=np.int64)  # bottom
            out[np.abs(xm - x1) < eps] = 1  # right
            out[np.abs(ym - y1) < eps] = 2  # top
            out[np.abs(xm - x0) < eps] = 3  # left
            return out

        patch_defs = patch_defs or [("bottom", BC_OUTLET), ("right", BC_OUTLET), ("top", BC_OUTLET),
                                    ("left", BC_OUTLET)]
    return build_foam_mesh(pts, cell_ptr, cell_pts, classify, patch_defs, renumber=renumber)


def periodic_quad_grid(nx, ny, x0=0.0, x1=1.0, y0=0.0, y1=1.0, renumber=True):
    """nx x ny quads on [x0,x1] x [y0,y1], periodic in both directions (no boundary faces).  The
    points of the last column and row are duplicates of the first, tied to them by the alias."""
    xs = np.linspace(x0, x1, nx + 1)
    ys = np.linspace(y0, y1, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel()], axis=1)
    I, J = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    alias = ((I % nx) * (ny + 1) + (J % ny)).ravel()
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    I = I.ravel()
    J = J.ravel()
    quads = np.stack([I * (ny + 1) + J, (I + 1) * (ny + 1) + J, (I + 1) * (ny + 1) + J + 1, I * (ny + 1) + J + 1],
                     axis=1)

    def classify(xm, ym):
        raise ValueError("a doubly periodic mesh has no boundary faces")

    return build_foam_mesh(pts, np.arange(0, 4 * quads.shape[0] + 1, 4), quads.ravel(), classify, [],
                           renumber=renumber, alias=alias, period=(x1 - x0, y1 - y0))


def wedge_quads(nx, ny, angle_deg, x_ramp=0.5, length=2.0, height=1.0, renumber=True):
    """Supersonic compression ramp: the channel [0, length] x [0, height] whose floor turns up by
    ``angle_deg`` at x = x_ramp; nx x ny quads, each column spanning floor to ceiling.  Patches:
    inflow x = 0 (label 6: its ghost keeps the inflow state given at set-up), outflow x = length
    (label 4), slip walls on floor and ceiling (label 2)."""
    xs = np.linspace(0.0, length, nx + 1)
    yb = np.where(xs > x_ramp, (xs - x_ramp) * np.tan(np.radians(angle_deg)), 0.0)
    if yb.max() >= 0.8 * height:
        raise ValueError("the ramp leaves less than a fifth of the channel height")
    eta = np.linspace(0.0, 1.0, ny + 1)
    X = np.repeat(xs[:, None], ny + 1, axis=1)
    Y = yb[:, None] + (height - yb[:, None]) * eta[None, :]
    pts = np.stack([X.ravel(), Y.ravel()], axis=1)
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    I = I.ravel()
    J = J.ravel()
    quads = np.stack([I * (ny + 1) + J, (I + 1) * (ny + 1) + J, (I + 1) * (ny + 1) + J + 1, I * (ny + 1) + J + 1],
                     axis=1)
    eps = 1e-9 * length

    def classify(xm, ym):
        out = np.full(xm.shape[0], 2, dtype=np.int64)  # walls
        out[np.abs(xm) < eps] = 0
        out[np.abs(xm - length) < eps] = 1
        return out

    return build_foam_mesh(pts, np.arange(0, 4 * quads.shape[0] + 1, 4), quads.ravel(), classify,
                           [("inflow", BC_FIXED_INITIAL), ("outflow", BC_OUTLET), ("walls", BC_SLIP)],
                           renumber=renumber)


def corner_flow(n=500):
    """The reference's cornerFlow case geometry (reference simulation/cornerFlow/cornerFlow_cuda/
    system/blockMeshDict:17-76): the unit square, inlet on x=0 above y=0.5 (label 5), slip walls on
    x=0 below y=0.5 and on y=0, y=1 (label 2), outlet on x=1 (label 4)."""
    eps = 1e-12

    def classify(xm, ym):
        out = np.full(xm.shape[0], 1, dtype=np.int64)  # obstacle
        out[(np.abs(xm) < eps) & (ym > 0.5)] = 0  # inlet
        out[np.abs(xm - 1.0) < eps] = 2  # outlet
        return out

    mesh = quad_grid(n, n, classify=classify,
                     patch_defs=[("inlet", BC_FIXED_VALUE2), ("obstacle", BC_SLIP), ("outlet", BC_OUTLET)])
    return mesh


def forward_step_triangles(n_points=1_000_000, jitter=0.3, seed=0, renumber=True):
    """Mach 3 forward-facing step: channel [0,3]x[0,1] with the step [0.6,3]x[0,0.2] removed,
    Delaunay triangulation of a seeded jittered point set (jitter * h) of about ``n_points``
    points.  Patches: inflow x=0 (label 3: p=1, U=(3,0), T=1, i.e. rho=1.4 at R=1/1.4),
    supersonic outflow x=3 (label 4), slip walls elsewhere (label 2)."""
    from scipy.spatial import Delaunay

    area = 3.0 * 1.0 - 2.4 * 0.2
    h0 = math.sqrt(area / n_points)
    k = max(1, int(round(0.2 / h0)))
    h = 0.2 / k
    nx = int(round(3.0 / h))
    ny = int(round(1.0 / h))
    xs = np.arange(nx + 1) * h
    ys = np.arange(ny + 1) * h
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    X = X.ravel()
    Y = Y.ravel()
    tol = 1e-9 * h
    solid = (X > 0.6 + tol) & (Y < 0.2 - tol)
    X = X[~solid]
    Y = Y[~solid]
    on_bnd = ((X < tol) | (X > 3.0 - tol) | (Y > 1.0 - tol) | (Y < tol)
              | ((np.abs(X - 0.6) < tol) & (Y <= 0.2 + tol)) | ((np.abs(Y - 0.2) < tol) & (X >= 0.6 - tol)))
    rng = np.random.default_rng(seed)
    d = rng.uniform(-jitter * h, jitter * h, size=(X.shape[0], 2))
    d[on_bnd] = 0.0
    pts = np.stack([X + d[:, 0], Y + d[:, 1]], axis=1)
    tri = Delaunay(pts).simplices.astype(np.int64)
    c = pts[tri].mean(axis=1)
    keep = ~((c[:, 0] > 0.6) & (c[:, 1] < 0.2))
    tri = tri[keep]
    p0 = pts[tri[:, 0]]
    p1 = pts[tri[:, 1]]
    p2 = pts[tri[:, 2]]
    cross = (p1[:, 0] - p0[:, 0]) * (p2[:, 1] - p0[:, 1]) - (p2[:, 0] - p0[:, 0]) * (p1[:, 1] - p0[:, 1])
    tri = tri[np.abs(cross) > 1e-6 * h * h]
    cross = cross[np.abs(cross) > 1e-6 * h * h]
    flip = cross < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    cell_ptr = np.arange(0, 3 * tri.shape[0] + 1, 3)
    eps = 1e-9 * h

    def classify(xm, ym):
        out = np.full(xm.shape[0], 2, dtype=np.int64)  # walls
        out[xm < eps] = 0
        out[xm > 3.0 - eps] = 1
        return out

    return build_foam_mesh(pts, cell_ptr, tri.ravel(), classify,
                           [("inflow", BC_FIXED_VALUE), ("outflow", BC_OUTLET), ("walls", BC_SLIP)],
                           renumber=renumber)


def riemann_mixed(n=1766, radius=0.3, seed=0, renumber=True):
    """Unit square of quads with the cells inside a central disk of ``radius`` split into seeded
    triangles: a conforming mixed quad/triangle mesh (about 4M cells at n=1766).  All sides are
    outlets (label 4)."""
    def tri_mask(xc, yc):
        return (xc - 0.5) ** 2 + (yc - 0.5) ** 2 < radius * radius

    return quad_grid(n, n, tri_mask=tri_mask, seed=seed, renumber=renumber)


# ---------------------------------------------------------------------------------- initial fields
GAMMA = 1.4
R_GAS = 1.0 / 1.4
CV_GAS = R_GAS / (GAMMA - 1.0)


def uniform_fields(mesh: FoamMesh, p, ux, uy, T):
    nc = mesh.n_cells
    nb = mesh.n_boundary_faces
    W = np.empty((nc, 4))
    W[:] = (p, ux, uy, T)
    Wb = np.empty((nb, 4))
    Wb[:] = (p, ux, uy, T)
    return W, Wb


def riemann_fields(mesh: FoamMesh, R=R_GAS):
    """Four-quadrant Riemann states (rho, u, v, p) about (0.5, 0.5); returns W=(p,Ux,Uy,T)."""
    c = mesh.cell_centres()
    x, y = c[:, 0], c[:, 1]
    q = np.where(x >= 0.5, np.where(y >= 0.5, 0, 3), np.where(y >= 0.5, 1, 2))
    states = np.array([[1.5, 0.0, 0.0, 1.5],
                       [0.5323, 1.206, 0.0, 0.3],
                       [0.138, 1.206, 1.206, 0.029],
                       [0.5323, 0.0, 1.206, 0.3]])
    s = states[q]
    W = np.stack([s[:, 3], s[:, 1], s[:, 2], s[:, 3] / (R * s[:, 0])], axis=1)
    bc = mesh.boundary_face_centres()
    own = mesh.owner[mesh.n_internal_faces:]
    Wb = W[own].copy()
    del bc
    return W, Wb


def vortex_fields(xy, strength=5.0, xc=5.0, yc=5.0, u0=1.0, v0=1.0, R=R_GAS, gamma=GAMMA):
    """Isentropic vortex on a free stream rho=1, u=v=1, p=1 (W=(p,Ux,Uy,T)); point values."""
    dx = xy[:, 0] - xc
    dy = xy[:, 1] - yc
    r2 = dx * dx + dy * dy
    f = strength / (2.0 * math.pi) * np.exp(0.5 * (1.0 - r2))
    u = u0 - f * dy
    v = v0 + f * dx
    Ttil = 1.0 - (gamma - 1.0) * strength ** 2 / (8.0 * gamma * math.pi ** 2) * np.exp(1.0 - r2)
    rho = Ttil ** (1.0 / (gamma - 1.0))
    p = rho ** gamma
    T = p / (R * rho)
    return np.stack([p, u, v, T], axis=1)


# Isentropic vortex workload.  The reference has no periodic patch type, so the vortex travels in
# a box wide enough that its perturbation at the outlet (label 4) boundary stays below 1e-10.
VORTEX_BOX = (-7.0, 9.0)  # square [-7, 9]^2; the vortex starts at (0, 0) and moves with (1, 1)


def vortex_box(n, renumber=True):
    """n x n quads on the vortex box, outlet (label 4) on every side."""
    lo, hi = VORTEX_BOX
    return quad_grid(n, n, lo, hi, lo, hi, renumber=renumber)


def conserved_from_primitive(W, R=R_GAS, Cv=CV_GAS):
    """(p, Ux, Uy, T) -> (rho, rho Ux, rho Uy, rho E) with E = Cv T + |U|^2 / 2."""
    p, u, v, T = W[:, 0], W[:, 1], W[:, 2], W[:, 3]
    rho = p / (R * T)
    return np.stack([rho, rho * u, rho * v, rho * (Cv * T + 0.5 * (u * u + v * v))], axis=1)


def primitive_from_conserved(U, R=R_GAS, Cv=CV_GAS):
    rho = U[:, 0]
    u = U[:, 1] / rho
    v = U[:, 2] / rho
    T = (U[:, 3] / rho - 0.5 * (u * u + v * v)) / Cv
    return np.stack([rho * R * T, u, v, T], axis=1)


def vortex_cell_averages(mesh: FoamMesh, quadrature, t, strength=5.0, R=R_GAS, gamma=GAMMA, centre=(0.0, 0.0)):
    """Cell averages of the conserved variables of the exact solution at time t (the vortex centre
    at centre + (t, t)), from Gauss points/weights (offsets, points, weights over cells first).  On a
    periodic mesh each point takes its nearest image of the vortex."""
    off, pts, w = quadrature
    nc = mesh.n_cells
    npts = int(off[nc])
    xc, yc = centre[0] + t, centre[1] + t
    p = pts[:npts].copy()
    for k, L in enumerate(mesh.period):
        if L > 0:
            c = (xc, yc)[k]
            p[:, k] = c + (p[:, k] - c - L * np.rint((p[:, k] - c) / L))
    W = vortex_fields(p, strength=strength, xc=xc, yc=yc, R=R, gamma=gamma)
    U = conserved_from_primitive(W, R=R, Cv=R / (gamma - 1.0)) * w[:npts, None]
    sums = np.add.reduceat(U, off[:nc], axis=0)
    wsum = np.add.reduceat(w[:npts], off[:nc])
    return sums / wsum[:, None]
