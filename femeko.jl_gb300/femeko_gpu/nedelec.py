"""Nedelec (Whitney) edge elements on the GPU: the vector-potential magnetostatics of
Magnetostatics/nedelec3D.jl and the element routines of src/FEM3D.jl:155-271.

The unknowns are the edges of a second-order tetrahedral mesh, numbered as
src/mesh.jl:168-183 does (``unique(t[5:10, :])`` in first-appearance order).  Local edge
e of an element joins its local vertices (1,2), (2,3), (3,1), (4,1), (3,4), (2,4)
(src/mesh.jl:603-630) and is used in that local orientation, as the reference does.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import _lib as L
from .mesh import MESH


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def nedelec_edges(mesh: MESH):
    """(edges 6 x nt, 0-based edge unknowns; ne)."""
    mids = np.asarray(mesh.t[4:10], dtype=np.int64)
    flat = mids.T.ravel()
    _, first = np.unique(flat, return_index=True)
    order = np.sort(first)
    rank = np.full(int(flat.max()) + 1, -1, dtype=np.int64)
    rank[flat[order]] = np.arange(order.size)
    return rank[mids].astype(np.int32), int(order.size)


class EdgeGPUMesh:
    """Owns one fg_mesh handle over the edges of a P2 tetrahedral mesh."""

    def __init__(self, mesh: MESH):
        if mesh.t.shape[0] != 10:
            raise ValueError("Nedelec elements need the edge (midpoint) rows of a P2 tetrahedral mesh")
        lib = L.lib()
        self.mesh = mesh
        self.edges, self.ne = nedelec_edges(mesh)
        self._p = _c(mesh.p.T, np.float64)
        self._t = _c(np.asarray(mesh.t[:4]).T, np.int32)
        self._e = _c(self.edges.T, np.int32)
        h = C.c_void_p()
        L.check(lib.fg_edge_mesh_create(L.ptr(self._p), mesh.nv, L.ptr(self._t), L.ptr(self._e), mesh.nt, self.ne, 0,
                                        C.byref(h)))
        self.h = h
        L.register_handle(self)
        nnz, mr = C.c_int64(), C.c_int32()
        L.check(lib.fg_mesh_nnz(h, C.byref(nnz), C.byref(mr)))
        self.nnz = nnz.value
        self.colptr = np.zeros(self.ne + 1, dtype=np.int64)
        self.rowval = np.zeros(self.nnz, dtype=np.int32)
        L.check(lib.fg_csc_pattern(h, L.ptr(self.colptr), L.ptr(self.rowval), 0))

    def csc(self, vals):
        return sp.csc_matrix((vals, self.rowval.copy(), self.colptr.copy()), shape=(self.ne, self.ne))

    def close(self):
        if getattr(self, "h", None) and not L._shutting_down:
            L.lib().fg_mesh_destroy(self.h)
        self.h = None
        L.unregister_handle(self)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def edge_mesh(mesh: MESH) -> EdgeGPUMesh:
    g = getattr(mesh, "_gpu_edge", None)
    if g is None or g.h is None:
        g = EdgeGPUMesh(mesh)
        object.__setattr__(mesh, "_gpu_edge", g)
    return g


def nedelecLocalStiffness(mesh: MESH):
    """``src/FEM3D.jl:155-191``: Ak (36 x nt, column k the 6 x 6 block)."""
    g = edge_mesh(mesh)
    Ak = np.zeros(36 * mesh.nt)
    L.check(L.lib().fg_nedelec_local_stiffness(g.h, L.ptr(Ak)))
    return Ak.reshape(mesh.nt, 36).T


def nedelecStiffness(mesh: MESH, nu=None):
    """Global curl-curl matrix with reluctance nu (nedelec3D.jl:168-178), ne x ne CSC."""
    g = edge_mesh(mesh)
    vals = np.zeros(g.nnz)
    nv_ = None if nu is None else _c(nu, np.float64)
    L.check(L.lib().fg_nedelec_stiffness(g.h, L.ptr(nv_), L.ptr(vals)))
    return g.csc(vals)


def nedelecTangentialStiffness(mesh: MESH, dnu, Bfield, B):
    """``src/FEM3D.jl:194-271`` (a zero |B| contributes 0)."""
    g = edge_mesh(mesh)
    vals = np.zeros(g.nnz)
    L.check(L.lib().fg_nedelec_tangent(g.h, L.ptr(_c(dnu, np.float64)), L.ptr(_c(np.asarray(Bfield).T, np.float64)),
                                       L.ptr(_c(B, np.float64)), L.ptr(vals)))
    return g.csc(vals)


def nedelec_load(mesh: MESH, Bext):
    """Load vector RHS_e = sum VE Bext.curlN_e (nedelec3D.jl:106-139)."""
    g = edge_mesh(mesh)
    rhs = np.zeros(g.ne)
    L.check(L.lib().fg_nedelec_load(g.h, L.ptr(_c(Bext, np.float64)), L.ptr(rhs)))
    return rhs


def nedelec_bfield(mesh: MESH, u):
    """B per element (3 x nt) and its norm from the edge values (nedelec3D.jl:190-221)."""
    g = edge_mesh(mesh)
    Bf, B = np.zeros(3 * mesh.nt), np.zeros(mesh.nt)
    L.check(L.lib().fg_nedelec_bfield(g.h, L.ptr(_c(u, np.float64)), L.ptr(Bf), L.ptr(B)))
    return Bf.reshape(mesh.nt, 3).T, B


def nedelec_linear(mesh: MESH, Bext, nu=None, precision="fp64", rtol=1e-10, maxiter=1_000_000):
    """A(nu) u = RHS(Bext) by Jacobi-PCG on the GPU (the first Newton step of
    nedelec3D.jl, u = 0 and At = 0); returns (u, Bfield 3 x nt, |B|, stats)."""
    from . import solve_opts
    g = edge_mesh(mesh)
    u = np.zeros(g.ne)
    Bf, B = np.zeros(3 * mesh.nt), np.zeros(mesh.nt)
    o = solve_opts(precision=precision, rtol=rtol, maxiter=maxiter)
    s = L.SolveStats()
    nv_ = None if nu is None else _c(nu, np.float64)
    st = L.lib().fg_nedelec_linear(g.h, L.ptr(nv_), L.ptr(_c(Bext, np.float64)), L.ptr(u), L.ptr(Bf), L.ptr(B),
                                   C.byref(o), C.byref(s))
    L.check(st, allow_not_converged=True)
    return u, Bf.reshape(mesh.nt, 3).T, B, L.stats_dict(s)


def nedelec_newton(mesh: MESH, Bext, curve_B, curve_nu, nonlinear=None, nu_lin=None, tol=1e-4, max_newton=100,
                   min_step=1e-4, precision="fp64", rtol=1e-10, maxiter=1_000_000, use_graph=1):
    """The Newton loop of Magnetostatics/nedelec3D.jl:149-231 on the GPU with the
    material curve nu(B) given as a table (not-a-knot cubic interpolant, as Dierckx's
    Spline1D(B, nu)).  nonlinear: element mask (default: ``mesh.InsideElements``).
    Returns (u, Bfield 3 x nt, |B|, nu, newton steps, stats)."""
    from . import solve_opts
    g = edge_mesh(mesh)
    if nonlinear is None:
        nonlinear = np.zeros(mesh.nt, dtype=np.uint8)
        nonlinear[np.asarray(mesh.InsideElements, dtype=np.int64)] = 1
    u = np.zeros(g.ne)
    Bf, B, nu = np.zeros(3 * mesh.nt), np.zeros(mesh.nt), np.zeros(mesh.nt)
    it = C.c_int32()
    o = solve_opts(precision=precision, rtol=rtol, maxiter=maxiter, use_graph=use_graph)
    s = L.SolveStats()
    nl_ = None if nu_lin is None else _c(nu_lin, np.float64)
    cb, cn = _c(curve_B, np.float64), _c(curve_nu, np.float64)
    st = L.lib().fg_nedelec_newton(g.h, L.ptr(_c(Bext, np.float64)), L.ptr(_c(nonlinear, np.uint8)), L.ptr(nl_),
                                   L.ptr(cb), L.ptr(cn), int(cb.size), float(tol), int(max_newton), float(min_step),
                                   L.ptr(u), L.ptr(Bf), L.ptr(B), L.ptr(nu), C.byref(it), C.byref(o), C.byref(s))
    L.check(st, allow_not_converged=True)
    d = L.stats_dict(s)
    d["short_inner_solves"] = s.pad_
    return u, Bf.reshape(mesh.nt, 3).T, B, nu, it.value, d
