"""Mesh files in the reference's text format, read into a ``MESH`` the GPU path takes.

``save2file`` (``src/geometry.jl:237-245``) writes an array with each row on one line
and the row's entries joined by ``" , "`` (a vector: one entry per line).
``Mesh``/``Mesh2D`` write a mesh this way when ``saveMesh`` is set
(``src/mesh.jl:233-242``, ``:385-394``): ``t.txt`` (npe x nt, 1-based), ``p.txt``
(3 x nv), ``surfaceT.txt`` (face nodes, 1-based, and the boundary id in the last row),
``InsideNodes.txt``, ``InsideElements.txt`` (1-based), ``VE.txt``, ``AE.txt`` and
``normal.txt``.  The reference writes these files and reads none of them back;
``load_mesh`` reads such a folder (a Gmsh mesh made elsewhere) and ``save_mesh`` writes
one in the same format.

The files carry no per-element region tags: ``elementID`` is rebuilt as 1 (the
container) with 2 on ``InsideElements``, and the Dirichlet nodes as the nodes of the
surface faces whose boundary id is in ``shell_id`` (for second-order meshes with the
midpoint nodes of those faces' edges, which ``surfaceT`` does not list).
"""
from __future__ import annotations

import os

import numpy as np

from .mesh import MESH, TET10_EDGES, TRI6_EDGES

FILES = ("t", "p", "InsideNodes", "surfaceT", "InsideElements", "VE", "AE", "normal")


def _fmt(x) -> str:
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    return repr(float(x))   # shortest text that reads back to the same double


def save2file(path: str, a) -> None:
    """One line per row of a 2-D array (one line per entry of a vector), entries
    joined by " , " (``src/geometry.jl:237-245``)."""
    a = np.asarray(a)
    rows = a.reshape(-1, 1) if a.ndim == 1 else a
    with open(path, "w") as f:
        for row in rows:
            f.write(" , ".join(_fmt(x) for x in row) + "\n")


def load2array(path: str, dtype=np.float64) -> np.ndarray:
    """The array a ``save2file`` text holds: rows x columns, or a vector when every
    line has one entry.  Julia's number texts (``1.0e-5``, ``-0.0``, ``Inf``, ``NaN``)
    read as Python floats do."""
    rows = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if line:
                rows.append([float(x) for x in line.split(",")])
    if not rows:
        return np.zeros(0, dtype=dtype)
    width = {len(r) for r in rows}
    if len(width) != 1:
        raise ValueError(f"{path}: rows of different lengths {sorted(width)}")
    a = np.array(rows, dtype=np.float64)
    if a.shape[1] == 1:
        a = a[:, 0]
    if np.issubdtype(np.dtype(dtype), np.integer):
        if not np.all(np.isfinite(a)) or np.any(a != np.round(a)):
            raise ValueError(f"{path}: entries are not integers")
        a = np.rint(a)
    return a.astype(dtype)


def save_mesh(folder: str, mesh: MESH) -> None:
    """The eight files of ``src/mesh.jl:233-242`` (1-based indices, as Julia holds them)."""
    os.makedirs(folder, exist_ok=True)
    st = mesh.surfaceT.copy()
    st[:-1] += 1
    data = {"t": mesh.t + 1, "p": mesh.p, "InsideNodes": mesh.InsideNodes + 1, "surfaceT": st,
            "InsideElements": mesh.InsideElements + 1, "VE": mesh.VE, "AE": mesh.AE, "normal": mesh.normal}
    for name in FILES:
        save2file(os.path.join(folder, name + ".txt"), data[name])


def load_mesh(folder: str, shell_id=(1,)) -> MESH:
    """A ``MESH`` from the files ``save_mesh`` (or the reference's ``saveMesh``) wrote."""
    def rd(name, dtype=np.float64):
        return load2array(os.path.join(folder, name + ".txt"), dtype)

    t = rd("t", np.int64)
    if t.ndim == 1:
        t = t.reshape(-1, 1)
    p = rd("p")
    if p.ndim == 1:
        p = p.reshape(-1, 1)
    npe = t.shape[0]
    if npe not in (3, 4, 6, 10):
        raise ValueError(f"t.txt: {npe} nodes per element (3, 4, 6 or 10 expected)")
    dim = 3 if npe in (4, 10) else 2
    nv, nt = p.shape[1], t.shape[1]
    t = t - 1
    if t.min() < 0 or t.max() >= nv:
        raise ValueError("t.txt: node index out of range")
    st = rd("surfaceT", np.int64)
    if st.ndim == 1:
        st = st.reshape(-1, 1)
    st[:-1] -= 1
    inside_el = rd("InsideElements", np.int64).reshape(-1) - 1
    inside_nd = rd("InsideNodes", np.int64).reshape(-1) - 1
    element_id = np.ones(nt, dtype=np.int32)
    element_id[inside_el] = 2
    outer = np.isin(st[-1], np.asarray(shell_id))
    boundary = np.unique(st[:-1, outer]).astype(np.int64)
    if npe in (6, 10):
        # second order: surfaceT holds the faces' vertices; their edges' midpoint
        # nodes (element rows after the vertices, in Gmsh's edge order) are boundary too
        edges = TET10_EDGES if npe == 10 else TRI6_EDGES
        nvert = dim + 1
        va = np.concatenate([t[a] for a, b in edges])
        vb = np.concatenate([t[b] for a, b in edges])
        mid = np.concatenate([t[nvert + e] for e in range(len(edges))])
        key = np.minimum(va, vb) * nv + np.maximum(va, vb)
        order = np.argsort(key, kind="stable")
        key, mid = key[order], mid[order]
        fv = st[:-1, outer]
        pairs = [(0, 1), (1, 2), (2, 0)] if fv.shape[0] == 3 else [(0, 1)]
        fkey = np.concatenate([np.minimum(fv[i], fv[j]) * nv + np.maximum(fv[i], fv[j]) for i, j in pairs])
        pos = np.searchsorted(key, fkey)
        if np.any(pos >= key.size) or np.any(key[np.minimum(pos, key.size - 1)] != fkey):
            raise ValueError("surfaceT.txt: a boundary edge is not an element edge")
        boundary = np.unique(np.concatenate([boundary, mid[pos]]))
    normal = rd("normal")
    if normal.ndim == 1:
        normal = normal.reshape(-1, 1)
    return MESH(order=2 if npe in (6, 10) else 1, dim=dim, p=p, t=t.astype(np.int32),
                surfaceT=st.astype(np.int32), elementID=element_id, InsideElements=inside_el.astype(np.int32),
                InsideNodes=inside_nd.astype(np.int32), VE=rd("VE").reshape(-1), AE=rd("AE").reshape(-1),
                normal=normal, shell_id=tuple(shell_id), boundary_nodes=boundary)
