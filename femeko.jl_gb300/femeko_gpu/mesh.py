"""Synthetic structured meshes that fill the fields of Femeko's ``MESH`` struct.

The reference builds every mesh through Gmsh (``src/mesh.jl:62-397``, ``Mesh`` and
``Mesh2D``).  Gmsh is not part of this library; these generators produce the same
fields for seeded structured meshes instead:

* ``p``          3 x nv float64, column-major (``src/mesh.jl:15``)
* ``t``          npe x nt int32 connectivity (``src/mesh.jl:18``); stored 0-based here,
                 ``t1`` gives the 1-based view Julia holds
* ``surfaceT``   (3|2 + 1) x ns int32, last row = boundary id (``src/mesh.jl:21``)
* ``elementID``, ``InsideElements``, ``InsideNodes`` (``src/mesh.jl:30-36``)
* ``VE``, ``AE``, ``normal`` (``src/mesh.jl:39-45``; ``elementVolume`` ``:484-505``,
  ``areaTriangle`` ``:474-481``, ``normalSurface`` ``:436-450``)
* ``nv``, ``nt``, ``ns``, ``nInside``, ``nInsideNodes``, ``shell_id``

3D meshes: the box [-L, L]^3 is cut into n^3 hex cells, each split into the 6 Kuhn
tetrahedra that share the cell diagonal (0,0,0)->(1,1,1).  Node (i, j, k) has id
i + N*(j + N*k) with N = n + 1.  Interior nodes are jittered uniformly in +-jitter*h
per axis with numpy's PCG64 generator seeded by ``seed``.  Second-order meshes add one
node per edge midpoint, in Gmsh's 10-node tetrahedron order (edges 01, 12, 20, 30, 32, 31).

2D meshes: the square [-L, L]^2 cut into n^2 cells, each split into 2 triangles, with
``p`` stored 3 x nv (z = 0) as Gmsh returns it (``src/mesh.jl:322-324``); second order
adds edge midpoints in Gmsh's 6-node triangle order (edges 01, 12, 20).
"""
from __future__ import annotations

from dataclasses import dataclass, field
import itertools

import numpy as np

MU0 = np.pi * 4e-7

# The six Kuhn tetrahedra of a unit cell: walk from corner (0,0,0) to (1,1,1)
# adding one axis at a time, in each of the 3! axis orders.
_KUHN_PERMS = list(itertools.permutations(range(3)))
# Gmsh local edge order for the 10-node tetrahedron and the 6-node triangle.
TET10_EDGES = ((0, 1), (1, 2), (2, 0), (3, 0), (3, 2), (3, 1))
TRI6_EDGES = ((0, 1), (1, 2), (2, 0))


@dataclass
class MESH:
    """Field-for-field mirror of ``mutable struct MESH`` (``src/mesh.jl:9-59``)."""

    order: int
    dim: int
    p: np.ndarray                 # 3 x nv float64
    t: np.ndarray                 # npe x nt int32, 0-based
    surfaceT: np.ndarray          # (nodes+1) x ns int32, 0-based nodes, last row boundary id
    elementID: np.ndarray         # nt int32 region tag (1 = container, 2.. = cells)
    InsideElements: np.ndarray    # 0-based element ids with elementID != 1
    InsideNodes: np.ndarray       # 0-based node ids touched by InsideElements
    VE: np.ndarray                # nt float64 element volume (area in 2D)
    AE: np.ndarray                # ns float64 surface element area (length in 2D)
    normal: np.ndarray            # 3 x ns (2 x ns in 2D) outward unit normals
    shell_id: tuple = (1,)
    boundary_nodes: np.ndarray = field(default=None)   # 0-based, sorted
    cells: int = 0                # cells per side of the structured generator
    half_width: float = 5.0

    @property
    def nv(self) -> int:
        return self.p.shape[1]

    @property
    def nt(self) -> int:
        return self.t.shape[1]

    @property
    def ns(self) -> int:
        return self.surfaceT.shape[1]

    @property
    def nInside(self) -> int:
        return int(self.InsideElements.size)

    @property
    def nInsideNodes(self) -> int:
        return int(self.InsideNodes.size)

    @property
    def npe(self) -> int:
        return self.t.shape[0]

    @property
    def t1(self) -> np.ndarray:
        """1-based connectivity, as Julia's ``mesh.t`` holds it."""
        return self.t + 1

    def centroids(self) -> np.ndarray:
        nvert = self.dim + 1
        return self.p[:, self.t[:nvert]].mean(axis=1)

    def dirichlet_mask(self) -> np.ndarray:
        m = np.zeros(self.nv, dtype=np.uint8)
        m[self.boundary_nodes] = 1
        return m


def element_volumes(p: np.ndarray, t: np.ndarray) -> np.ndarray:
    """|AB . (AC x AD)| / 6 per element (``src/mesh.jl:484-505``)."""
    a = p[:, t[0]]
    ab = p[:, t[1]] - a
    ac = p[:, t[2]] - a
    ad = p[:, t[3]] - a
    cr = np.cross(ac.T, ad.T).T
    return np.abs((ab * cr).sum(axis=0)) / 6.0


def triangle_areas(p: np.ndarray, t: np.ndarray) -> np.ndarray:
    """Planar triangle area from x, y (the 2D ``VE`` of ``Mesh2D``)."""
    a = p[:2, t[0]]
    u = p[:2, t[1]] - a
    v = p[:2, t[2]] - a
    return 0.5 * np.abs(u[0] * v[1] - u[1] * v[0])


def _surface_from_faces(p, faces):
    """AE and outward normals of boundary triangles (``src/mesh.jl:436-481``)."""
    p1, p2, p3 = (p[:, faces[i]] for i in range(3))
    n = np.cross((p2 - p1).T, (p3 - p1).T).T
    nn = np.sqrt((n * n).sum(axis=0))
    return 0.5 * nn, n / nn


def _edge_midpoints(t_vert, edges_local, nv):
    """Unique edges of the elements; returns (edge id per element-edge, endpoints)."""
    e = np.stack([np.sort(np.stack([t_vert[a], t_vert[b]]), axis=0) for a, b in edges_local], axis=1)
    # e: 2 x nedge_local x nt
    key = e[0].astype(np.int64) * nv + e[1]
    uniq, inv = np.unique(key.ravel(), return_inverse=True)
    ends = np.stack([uniq // nv, uniq % nv]).astype(np.int64)
    return inv.reshape(key.shape).astype(np.int64), ends


def box_tet_mesh(n: int, seed: int = 0, jitter: float = 0.1, half_width: float = 5.0,
                 order: int = 1, plate=((-1.0, 1.0), (-0.5, 0.5), (-0.25, 0.25))) -> MESH:
    """Structured Kuhn-tet mesh of [-L, L]^3 with n^3 cells (6 n^3 tets, (n+1)^3 vertices).

    Elements whose centroid lies inside the axis-aligned ``plate`` box get elementID 2
    (the reference's material cell), all others elementID 1 (the container).
    """
    N = n + 1
    h = 2.0 * half_width / n
    g = np.arange(N, dtype=np.float64) * h - half_width
    kk, jj, ii = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
    p = np.stack([g[ii], g[jj], g[kk]])
    interior = (ii > 0) & (ii < n) & (jj > 0) & (jj < n) & (kk > 0) & (kk < n)
    rng = np.random.Generator(np.random.PCG64(seed))
    jit = rng.uniform(-jitter * h, jitter * h, size=(3, N ** 3))
    p[:, interior] += jit[:, interior]

    ck, cj, ci = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    base = np.stack([ci, cj, ck])                    # 3 x ncell
    tets = []
    for perm in _KUHN_PERMS:
        cur = base.copy()
        verts = [cur[0] + N * (cur[1] + N * cur[2])]
        for ax in perm:
            cur = cur.copy()
            cur[ax] += 1
            verts.append(cur[0] + N * (cur[1] + N * cur[2]))
        tets.append(np.stack(verts))                 # 4 x ncell
    # element id = 6*cell + perm
    t = np.ascontiguousarray(np.stack(tets, axis=2).reshape(4, -1)).astype(np.int64)

    # Boundary faces: faces of boundary cells that lie on the box surface.
    bcell = (ci == 0) | (ci == n - 1) | (cj == 0) | (cj == n - 1) | (ck == 0) | (ck == n - 1)
    bel = (np.repeat(bcell, 6))
    tb = t[:, bel]
    faces = []
    for drop in range(4):
        keep = [a for a in range(4) if a != drop]
        f = tb[keep]
        opp = tb[drop]
        fi, fj, fk = f % N, (f // N) % N, f // (N * N)
        on = np.zeros(f.shape[1], dtype=bool)
        for coord in (fi, fj, fk):
            for val in (0, n):
                on |= (coord == val).all(axis=0)
        sel = on
        f = f[:, sel]
        opp = opp[sel]
        # orient outward: normal must point away from the opposite vertex
        p1, p2, p3 = p[:, f[0]], p[:, f[1]], p[:, f[2]]
        nrm = np.cross((p2 - p1).T, (p3 - p1).T).T
        flip = (nrm * (p[:, opp] - p1)).sum(axis=0) > 0
        f[[1, 2]] = np.where(flip, f[[2, 1]], f[[1, 2]])
        faces.append(f)
    faces = np.concatenate(faces, axis=1)
    # deterministic order
    faces = faces[:, np.lexsort(np.sort(faces, axis=0)[::-1])]
    ns = faces.shape[1]
    AE, normal = _surface_from_faces(p, faces)
    surfaceT = np.vstack([faces, np.ones((1, ns), dtype=np.int64)]).astype(np.int32)

    boundary = np.flatnonzero(~interior).astype(np.int32)

    cen = p[:, t].mean(axis=1)
    (x0, x1), (y0, y1), (z0, z1) = plate
    inside = ((cen[0] > x0) & (cen[0] < x1) & (cen[1] > y0) & (cen[1] < y1)
              & (cen[2] > z0) & (cen[2] < z1))
    elementID = np.where(inside, 2, 1).astype(np.int32)
    inside_el = np.flatnonzero(inside).astype(np.int32)
    inside_nodes = np.unique(t[:, inside_el]).astype(np.int32)

    VE = element_volumes(p, t)
    tt = t
    if order == 2:
        nvv = p.shape[1]
        eid, ends = _edge_midpoints(t, TET10_EDGES, nvv)
        mids = 0.5 * (p[:, ends[0]] + p[:, ends[1]])
        p = np.hstack([p, mids])
        tt = np.vstack([t, nvv + eid])
        # boundary midpoints are boundary nodes
        # a midpoint is a boundary node when its edge lies in a face of the box
        on = np.zeros(mids.shape[1], dtype=bool)
        for ax in range(3):
            for val in (0, n):
                c0 = (ends[0] // (N ** ax)) % N
                c1 = (ends[1] // (N ** ax)) % N
                on |= (c0 == val) & (c1 == val)
        boundary = np.concatenate([boundary, (nvv + np.flatnonzero(on)).astype(np.int32)])
        inside_nodes = np.unique(tt[:, inside_el]).astype(np.int32)
    return MESH(order=order, dim=3, p=np.ascontiguousarray(p), t=np.ascontiguousarray(tt.astype(np.int32)),
                surfaceT=surfaceT, elementID=elementID, InsideElements=inside_el,
                InsideNodes=inside_nodes, VE=VE, AE=AE, normal=normal, shell_id=(1,),
                boundary_nodes=np.sort(boundary).astype(np.int32), cells=n, half_width=half_width)


def box_tri_mesh(n: int, seed: int = 0, jitter: float = 0.1, half_width: float = 5.0,
                 order: int = 1, inset=((-1.0, 1.0), (-0.5, 0.5))) -> MESH:
    """Structured triangle mesh of [-L, L]^2: n^2 cells, each cut along its (0,0)-(1,1) diagonal."""
    N = n + 1
    h = 2.0 * half_width / n
    g = np.arange(N, dtype=np.float64) * h - half_width
    jj, ii = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    p = np.stack([g[ii], g[jj], np.zeros(N * N)])
    interior = (ii > 0) & (ii < n) & (jj > 0) & (jj < n)
    rng = np.random.Generator(np.random.PCG64(seed))
    jit = rng.uniform(-jitter * h, jitter * h, size=(2, N * N))
    p[:2, interior] += jit[:, interior]
    cj, ci = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    v00 = ci + N * cj
    v10 = v00 + 1
    v01 = v00 + N
    v11 = v00 + N + 1
    t = np.stack([np.stack([v00, v10, v11]), np.stack([v00, v11, v01])], axis=2).reshape(3, -1).astype(np.int64)
    # boundary edges, counter-clockwise so that (dy, -dx) is outward
    edges = []
    for c in range(n):
        edges.append((c, c + 1))                          # bottom, left->right
        edges.append((n + N * c, n + N * (c + 1)))        # right, bottom->top
        edges.append((N * n + c + 1, N * n + c))          # top, right->left
        edges.append((N * (c + 1), N * c))                # left, top->bottom
    edges = np.array(edges, dtype=np.int64).T
    d = p[:2, edges[1]] - p[:2, edges[0]]
    AE = np.sqrt((d * d).sum(axis=0))
    normal = np.stack([d[1], -d[0]]) / AE
    surfaceT = np.vstack([edges, np.ones((1, edges.shape[1]), dtype=np.int64)]).astype(np.int32)
    boundary = np.flatnonzero(~interior).astype(np.int32)
    cen = p[:, t].mean(axis=1)
    (x0, x1), (y0, y1) = inset
    inside = (cen[0] > x0) & (cen[0] < x1) & (cen[1] > y0) & (cen[1] < y1)
    elementID = np.where(inside, 2, 1).astype(np.int32)
    inside_el = np.flatnonzero(inside).astype(np.int32)
    VE = triangle_areas(p, t)
    tt = t
    if order == 2:
        nvv = p.shape[1]
        eid, ends = _edge_midpoints(t, TRI6_EDGES, nvv)
        mids = 0.5 * (p[:, ends[0]] + p[:, ends[1]])
        p = np.hstack([p, mids])
        tt = np.vstack([t, nvv + eid])
        on = np.zeros(mids.shape[1], dtype=bool)
        for ax in range(2):
            for val in (0, n):
                c0 = (ends[0] // (N ** ax)) % N
                c1 = (ends[1] // (N ** ax)) % N
                on |= (c0 == val) & (c1 == val)
        boundary = np.concatenate([boundary, (nvv + np.flatnonzero(on)).astype(np.int32)])
    inside_nodes = np.unique(tt[:, inside_el]).astype(np.int32)
    return MESH(order=order, dim=2, p=np.ascontiguousarray(p), t=np.ascontiguousarray(tt.astype(np.int32)),
                surfaceT=surfaceT, elementID=elementID, InsideElements=inside_el,
                InsideNodes=inside_nodes, VE=VE, AE=AE, normal=normal, shell_id=(1,),
                boundary_nodes=np.sort(boundary).astype(np.int32), cells=n, half_width=half_width)


def surface_faces6(mesh) -> np.ndarray:
    """6 x ns face nodes of a P2 tetrahedral mesh's surface triangles, in the order of
    the reference's P2 ``surfaceT`` rows 1-6: the three vertices, then the midpoints of
    edges 12, 23 and 31 (``src/FEM3D.jl:300-322`` reads them so).  The midpoints are
    found among the elements' edge nodes."""
    if mesh.t.shape[0] != 10:
        raise ValueError("surface_faces6: P2 tetrahedra only")
    t = np.asarray(mesh.t, dtype=np.int64)
    nv = mesh.nv
    va = np.concatenate([t[a] for a, b in TET10_EDGES])
    vb = np.concatenate([t[b] for a, b in TET10_EDGES])
    mid = np.concatenate([t[4 + e] for e in range(len(TET10_EDGES))])
    key = np.minimum(va, vb) * nv + np.maximum(va, vb)
    order = np.argsort(key, kind="stable")
    key, mid = key[order], mid[order]
    fv = np.asarray(mesh.surfaceT[:3], dtype=np.int64)
    out = np.zeros((6, fv.shape[1]), dtype=np.int32)
    out[:3] = fv
    for r, (i, j) in enumerate(((0, 1), (1, 2), (2, 0))):
        fk = np.minimum(fv[i], fv[j]) * nv + np.maximum(fv[i], fv[j])
        pos = np.minimum(np.searchsorted(key, fk), key.size - 1)
        if np.any(key[pos] != fk):
            raise ValueError("surface_faces6: a surface edge is not an element edge")
        out[3 + r] = mid[pos]
    return out


def surface_lines3(mesh) -> np.ndarray:
    """3 x ns boundary-edge nodes of a P2 triangle mesh in the order of the reference's
    P2 ``surfaceT`` rows 1-3 (Gmsh's 3-node line: the two vertices, then the midpoint),
    which ``src/FEM2D.jl:394-419`` reads.  The midpoints are found among the elements'
    edge nodes."""
    if mesh.t.shape[0] != 6:
        raise ValueError("surface_lines3: P2 triangles only")
    t = np.asarray(mesh.t, dtype=np.int64)
    nv = mesh.nv
    va = np.concatenate([t[a] for a, b in TRI6_EDGES])
    vb = np.concatenate([t[b] for a, b in TRI6_EDGES])
    mid = np.concatenate([t[3 + e] for e in range(len(TRI6_EDGES))])
    key = np.minimum(va, vb) * nv + np.maximum(va, vb)
    order = np.argsort(key, kind="stable")
    key, mid = key[order], mid[order]
    ev = np.asarray(mesh.surfaceT[:2], dtype=np.int64)
    fk = np.minimum(ev[0], ev[1]) * nv + np.maximum(ev[0], ev[1])
    pos = np.minimum(np.searchsorted(key, fk), key.size - 1)
    if np.any(key[pos] != fk):
        raise ValueError("surface_lines3: a boundary edge is not an element edge")
    return np.vstack([ev, mid[pos][None, :]]).astype(np.int32)


def surface_faces_p2(mesh) -> np.ndarray:
    """The P2 boundary faces the boundary mass reads: ``surface_faces6`` for
    tetrahedra, ``surface_lines3`` for triangles."""
    return surface_faces6(mesh) if mesh.t.shape[0] == 10 else surface_lines3(mesh)
