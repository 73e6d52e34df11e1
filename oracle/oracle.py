"""ctypes bindings for the CPU oracle (``femeko_oracle.c``).

TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.  Nothing in
the GPU library imports this module.  Parity of the oracle against reference outputs is
UNPINNED (no Julia and no Eigen to run the reference); it is pinned to analytic known
answers instead (``tests/test_oracle.py``, ``tests/golden/``).

All index arrays are 0-based.  Sparse results come back as ``scipy.sparse.csc_matrix``
(the reference's SparseMatrixCSC layout).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfemeko_oracle.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_bp = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_vp = C.c_void_p

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.or_version.restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        L.or_get_threads.restype = C.c_int
        L.or_element_volume.restype = C.c_double
        L.or_element_volume.argtypes = [_dp, _ip]
        L.or_element_volumes.argtypes = [_dp, _ip, C.c_long, _dp]
        L.or_area_triangle.restype = C.c_double
        L.or_area_triangle.argtypes = [_dp, _ip]
        L.or_abcd.argtypes = [_dp, _ip, C.c_int, _dp]
        L.or_abc.argtypes = [_dp, _ip, C.c_int, _dp]
        L.or_local_stiffness.argtypes = [_dp, _ip, C.c_long, _dp, _vp, _dp]
        csc_out = [_lp, _ip, _dp]
        L.or_assemble_csc.restype = C.c_long
        L.or_assemble_csc.argtypes = [C.c_int, C.c_long, C.c_int, _ip, _dp, C.c_int] + csc_out
        L.or_stiffness.restype = C.c_long
        L.or_stiffness.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _vp, C.c_int] + csc_out
        L.or_mass.restype = C.c_long
        L.or_mass.argtypes = [_ip, C.c_int, C.c_long, _dp, C.c_int] + csc_out
        L.or_tangent.restype = C.c_long
        L.or_tangent.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _dp, _dp, C.c_int] + csc_out
        L.or_stiffness2d.restype = C.c_long
        L.or_stiffness2d.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _vp, C.c_int] + csc_out
        L.or_mass2d.restype = C.c_long
        L.or_mass2d.argtypes = [_ip, C.c_int, C.c_long, _dp, C.c_int] + csc_out
        L.or_p2_stiffness.restype = C.c_long
        L.or_p2_stiffness.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _vp, C.c_int] + csc_out
        L.or_p2_mass.restype = C.c_long
        L.or_p2_mass.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _vp, C.c_int] + csc_out
        L.or_p2_convection.restype = C.c_long
        L.or_p2_convection.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _dp, _vp, C.c_int] + csc_out
        L.or_p2_convection2d.restype = C.c_long
        L.or_p2_convection2d.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _dp] + csc_out
        L.or_nedelec_local.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _vp, C.c_int, _vp, _vp, _vp, _dp]
        L.or_nedelec_load.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _ip, _dp, _dp]
        L.or_nedelec_bfield.argtypes = [_dp, _ip, C.c_int, C.c_long, _ip, _dp, _dp, _dp]
        L.or_p2_stiffness2d.restype = C.c_long
        L.or_p2_stiffness2d.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _vp, C.c_int] + csc_out
        L.or_p2_mass2d.restype = C.c_long
        L.or_p2_mass2d.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp] + csc_out
        L.or_lagrange.argtypes = [_ip, C.c_int, C.c_long, _dp, _dp]
        L.or_demag_field.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _bp, _dp, C.c_double, C.c_int, _dp, _dp,
                                     C.POINTER(C.c_int)]
        L.or_demag_field.restype = C.c_int
        L.or_boundary_integral.argtypes = [_ip, C.c_long, C.c_int, _dp, _dp, _dp, _ip, C.c_int, _dp]
        L.or_spmv.argtypes = [C.c_int, _lp, _ip, _dp, _dp, _dp]
        L.or_pcg.restype = C.c_int
        L.or_pcg.argtypes = [C.c_int, _lp, _ip, _dp, _dp, _dp, _vp, C.c_double, C.c_int, C.POINTER(C.c_double)]
        L.or_hfield.argtypes = [_dp, _ip, C.c_long, _dp, C.c_int, _dp]
        L.or_froehlich.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_energy.restype = C.c_double
        L.or_energy.argtypes = [_dp, _dp, C.c_long, _vp, _dp, C.c_double, C.c_double]
        L.or_newton.restype = C.c_int
        L.or_newton.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _bp, _bp, _dp, C.c_double, C.c_double,
                                C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                C.c_double, C.c_int, _dp, _dp, _dp, _dp]
        L.or_linear_magnetostatics.restype = C.c_int
        L.or_linear_magnetostatics.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _bp, _dp, C.c_double, C.c_int,
                                               _dp, _vp, C.POINTER(C.c_int)]
        L.or_heat_be.restype = C.c_int
        L.or_heat_be.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _bp, _dp, C.c_double, C.c_double, C.c_int,
                                 C.c_double, C.c_int, _dp, C.c_int, _vp, C.POINTER(C.c_int)]
        L.or_objective_hx.restype = C.c_double
        L.or_objective_hx.argtypes = [_dp, _ip, C.c_long, _dp, _bp, _dp]
        L.or_adjoint.restype = C.c_int
        L.or_adjoint.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _bp, _bp, _dp, _vp, _vp, _dp, C.c_double,
                                 C.c_int, _dp, _dp]
        L.or_newton_sample.argtypes = [_dp, _ip, C.c_int, C.c_long, _dp, _bp, _bp, _dp, C.c_double, C.c_double,
                                       _dp, C.c_int, _dp]
        _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _pt(mesh):
    """p (3 x nv) and t (npe x nt) as the column-major buffers the C code expects."""
    p = _c(mesh.p.T, np.float64)           # nv x 3 row-major == 3 x nv column-major
    t = _c(mesh.t.T, np.int32)             # nt x npe row-major == npe x nt column-major
    return p, t


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _csc(nv, nnz, cp, ri, v):
    return sp.csc_matrix((v[:nnz].copy(), ri[:nnz].copy(), cp.copy()), shape=(nv, nv))


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def get_threads() -> int:
    return lib().or_get_threads()


def element_volumes(mesh):
    p, t = _pt(mesh)
    VE = np.zeros(mesh.nt)
    lib().or_element_volumes(p, t, mesh.nt, VE)
    return VE


def abcd(mesh, k: int, a: int):
    p, t = _pt(mesh)
    out = np.zeros(4)
    lib().or_abcd(p, _c(t[k], np.int32), int(t[k, a]), out)
    return out


def _assemble(fn, mesh, npe, *args, drop_zeros=None):
    nv, nt = mesh.nv, mesh.nt
    m = npe * npe * nt
    cp = np.zeros(nv + 1, dtype=np.int64)
    ri = np.zeros(m, dtype=np.int32)
    v = np.zeros(m)
    extra = () if drop_zeros is None else (int(drop_zeros),)
    nnz = fn(*args, *extra, cp, ri, v)
    return _csc(nv, nnz, cp, ri, v)


def stiffnessMatrix(mesh, f=None, drop_zeros=False):
    """``src/FEM3D.jl:40-56``."""
    p, t = _pt(mesh)
    fv = None if f is None else _c(f, np.float64)
    return _assemble(lib().or_stiffness, mesh, 4, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), _ptr(fv),
                     drop_zeros=drop_zeros)


def localStiffnessMatrix(mesh, f=None):
    """``src/FEM3D.jl:59-76``: 16 x nt, pass order n = 4 i + j."""
    p, t = _pt(mesh)
    fv = None if f is None else _c(f, np.float64)
    Ak = np.zeros(16 * mesh.nt)
    lib().or_local_stiffness(p, t, mesh.nt, _c(mesh.VE, np.float64), _ptr(fv), Ak)
    return Ak.reshape(mesh.nt, 16).T


def massMatrix(mesh, drop_zeros=False):
    """``src/FEM3D.jl:466-492``."""
    _, t = _pt(mesh)
    return _assemble(lib().or_mass, mesh, 4, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), drop_zeros=drop_zeros)


def tangentialStiffnessMatrix(mesh, H_vec, dmu, drop_zeros=False):
    """``src/FEM3D.jl:79-119``; H_vec is 3 x nt."""
    p, t = _pt(mesh)
    return _assemble(lib().or_tangent, mesh, 4, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64),
                     _c(np.asarray(H_vec).T, np.float64), _c(dmu, np.float64), drop_zeros=drop_zeros)


def stiffnessMatrix2D(mesh, mu=None, drop_zeros=False):
    """``src/FEM2D.jl:48-76``."""
    p, t = _pt(mesh)
    mv = None if mu is None else _c(mu, np.float64)
    return _assemble(lib().or_stiffness2d, mesh, 3, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), _ptr(mv),
                     drop_zeros=drop_zeros)


def massMatrix2D(mesh, drop_zeros=False):
    """``src/FEM2D.jl:139-161``."""
    _, t = _pt(mesh)
    return _assemble(lib().or_mass2d, mesh, 3, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), drop_zeros=drop_zeros)


def quadraticStiffnessMatrix(mesh, mu=None, shift=True):
    """``src/FEM3D.jl:324-395`` (the basis solve in element-shifted coordinates by default)."""
    p, t = _pt(mesh)
    mv = None if mu is None else _c(mu, np.float64)
    return _assemble(lib().or_p2_stiffness, mesh, 10, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), _ptr(mv),
                     int(shift))


def quadraticMassMatrix(mesh, F=None, full_phi=False):
    """``src/FEM3D.jl:494-561``; full_phi=False reproduces the reference's linear-part-only phi."""
    p, t = _pt(mesh)
    fv = None if F is None else _c(F, np.float64)
    return _assemble(lib().or_p2_mass, mesh, 10, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), _ptr(fv),
                     int(full_phi))


def quadraticConvectionMatrix(mesh, u, F=None, full_phi=False):
    """``src/FEM3D.jl:563-648``; u is the nodal velocity (3 x nv)."""
    p, t = _pt(mesh)
    uv = _c(np.asarray(u, dtype=np.float64).T, np.float64)
    fv = None if F is None else _c(F, np.float64)
    return _assemble(lib().or_p2_convection, mesh, 10, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), uv,
                     _ptr(fv), int(full_phi))


# src/FEM3D.jl:303-308: the P2 triangle mass, nodes (v1, v2, v3, m12, m23, m31), times 180.
_FACE_MK = np.array([[6, -1, -1, 0, -4, 0],
                     [-1, 6, -1, 0, 0, -4],
                     [-1, -1, 6, -4, 0, 0],
                     [0, 0, -4, 32, 16, 16],
                     [-4, 0, 0, 16, 32, 16],
                     [0, -4, 0, 16, 16, 32]], dtype=np.float64)


def quadraticConvectionMatrix2D(mesh, u):
    """``src/FEM2D.jl:231-319``; u is the nodal velocity (2 or 3 x nv)."""
    p, t = _pt(mesh)
    u = np.asarray(u, dtype=np.float64)
    u3 = np.vstack([u[:2], np.zeros((1, u.shape[1]))])
    return _assemble(lib().or_p2_convection2d, mesh, 6, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64),
                     _c(u3.T, np.float64))


# src/FEM2D.jl:397-399: the 3-node line mass, by position in surfaceT rows 1-3, times 30.
_LINE_MK = np.array([[4, 2, -1], [2, 16, 2], [-1, 2, 4]], dtype=np.float64)


def quadraticMassMatrix1D(mesh, faces3, h=None):
    """``src/FEM2D.jl:394-419``: M[nds[i], nds[j]] += AE[s] Mk[i,j] h[s] over the
    boundary lines (faces3: 3 x ns, 0-based), Mk = (1/30) c."""
    ns = faces3.shape[1]
    h = np.ones(ns) if h is None else np.asarray(h, dtype=np.float64)
    Mk = (1.0 / 30.0) * _LINE_MK
    rows = np.repeat(faces3, 3, axis=0)
    cols = np.tile(faces3, (3, 1))
    vals = (np.asarray(mesh.AE[:ns])[None, :] * Mk.reshape(9, 1)) * h[None, :]
    return sp.csc_matrix((vals.ravel(), (rows.ravel(), cols.ravel())), shape=(mesh.nv, mesh.nv))


def quadraticBoundaryMassMatrix(mesh, faces6, F=None):
    """``src/FEM3D.jl:300-322``: M[nds[i], nds[j]] += AE[s] Mk[i,j] F[s] over the
    surface faces (faces6: 6 x ns, 0-based), Mk = (1/180) c."""
    ns = faces6.shape[1]
    F = np.ones(ns) if F is None else np.asarray(F, dtype=np.float64)
    Mk = (1.0 / 180.0) * _FACE_MK
    rows = np.repeat(faces6, 6, axis=0)            # (36, ns): row node of entry (i, j)
    cols = np.tile(faces6, (6, 1))                 # (36, ns): column node
    vals = (np.asarray(mesh.AE[:ns])[None, :] * Mk.reshape(36, 1)) * F[None, :]
    return sp.csc_matrix((vals.ravel(), (rows.ravel(), cols.ravel())), shape=(mesh.nv, mesh.nv))


def transport_be(mesh, T0, rhoCp, kappa, u, dt, nsteps, faces6=None, face_F=None, full_phi=True):
    """``Transport/main3D.jl:155-213``: LM = M + dt (A + R + C) and nsteps direct
    solves T = LM \\ (M T) (scipy's sparse LU standing in for Julia's ``\\``).
    Returns the list of fields after each step."""
    import scipy.sparse.linalg as spla
    if mesh.t.shape[0] == 6:
        # Transport/main2D.jl:162-190: M, A(epsi), C(u), R = quadraticMassMatrix1D(intakeBC)
        M = quadraticMassMatrix2D(mesh)
        A = quadraticStiffnessMatrix2D(mesh, kappa)
        Cm = quadraticConvectionMatrix2D(mesh, u)
        R = (sp.csc_matrix((mesh.nv, mesh.nv)) if face_F is None
             else quadraticMassMatrix1D(mesh, faces6, face_F))
    else:
        M = quadraticMassMatrix(mesh, rhoCp, full_phi=full_phi)
        A = quadraticStiffnessMatrix(mesh, kappa)
        Cm = quadraticConvectionMatrix(mesh, u, rhoCp, full_phi=full_phi)
        R = sp.csc_matrix((mesh.nv, mesh.nv)) if face_F is None else quadraticBoundaryMassMatrix(mesh, faces6, face_F)
    LM = (M + dt * (A + R + Cm)).tocsc()
    lu = spla.splu(LM)
    T = np.asarray(T0, dtype=np.float64).copy()
    out = []
    for _ in range(nsteps):
        T = lu.solve(M @ T)
        out.append(T.copy())
    return out


def nedelec_edges(mesh):
    """Edge unknowns of a P2 tetrahedral mesh as src/mesh.jl:168-183 numbers them:
    ``unique(t[5:10, :])`` in first-appearance order (element by element) mapped to
    1..ne (here 0..ne-1).  Returns (edges 6 x nt, ne)."""
    mids = np.asarray(mesh.t[4:10], dtype=np.int64)
    flat = mids.T.ravel()
    _, first = np.unique(flat, return_index=True)
    order = np.sort(first)
    rank = np.full(int(flat.max()) + 1, -1, dtype=np.int64)
    rank[flat[order]] = np.arange(order.size)
    return rank[mids].astype(np.int32), int(order.size)


def _ned_args(mesh):
    p = _c(mesh.p.T, np.float64)
    t4 = _c(np.asarray(mesh.t[:4]).T, np.int32)
    return p, t4


def nedelecLocalStiffness(mesh, nu=None):
    """``src/FEM3D.jl:155-191``: Ak (36 x nt; column k the 6 x 6 block row-major)."""
    p, t4 = _ned_args(mesh)
    Ak = np.zeros(36 * mesh.nt)
    nv_ = None if nu is None else _c(nu, np.float64)
    lib().or_nedelec_local(p, t4, 4, mesh.nt, _c(mesh.VE, np.float64), _ptr(nv_), 0, None, None, None, Ak)
    return Ak.reshape(mesh.nt, 36).T


def _ned_global(mesh, Ak, edges, ne):
    e = _c(edges.T, np.int32)
    m = 36 * mesh.nt
    cp, ri, v = np.zeros(ne + 1, dtype=np.int64), np.zeros(m, dtype=np.int32), np.zeros(m)
    V = _c(np.asarray(Ak).T, np.float64)
    nnz = lib().or_assemble_csc(ne, mesh.nt, 6, e, V, 0, cp, ri, v)
    return _csc(ne, nnz, cp, ri, v)


def nedelecStiffness(mesh, nu=None):
    """Global curl-curl matrix sum sparse(edge_i, edge_j, Ak .* nu) (nedelec3D.jl:168-178)."""
    edges, ne = nedelec_edges(mesh)
    return _ned_global(mesh, nedelecLocalStiffness(mesh, nu), edges, ne)


def nedelecTangentialStiffness(mesh, dnu, Bfield, B):
    """``src/FEM3D.jl:194-271`` (0 where |B| = 0)."""
    edges, ne = nedelec_edges(mesh)
    p, t4 = _ned_args(mesh)
    Ak = np.zeros(36 * mesh.nt)
    lib().or_nedelec_local(p, t4, 4, mesh.nt, _c(mesh.VE, np.float64), None, 1, _ptr(_c(dnu, np.float64)),
                           _ptr(_c(np.asarray(Bfield).T, np.float64)), _ptr(_c(B, np.float64)), Ak)
    return _ned_global(mesh, Ak.reshape(mesh.nt, 36).T, edges, ne)


def nedelec_load(mesh, Bext):
    edges, ne = nedelec_edges(mesh)
    p, t4 = _ned_args(mesh)
    rhs = np.zeros(ne)
    lib().or_nedelec_load(p, t4, 4, mesh.nt, _c(mesh.VE, np.float64), _c(edges.T, np.int32),
                          _c(Bext, np.float64), rhs)
    return rhs


def nedelec_bfield(mesh, u):
    edges, _ = nedelec_edges(mesh)
    p, t4 = _ned_args(mesh)
    Bf, Bn = np.zeros(3 * mesh.nt), np.zeros(mesh.nt)
    lib().or_nedelec_bfield(p, t4, 4, mesh.nt, _c(edges.T, np.int32), _c(u, np.float64), Bf, Bn)
    return Bf.reshape(mesh.nt, 3).T, Bn


def fd_gradient(x, y):
    """``src/FEM.jl:66-92``: one-sided differences at the ends, central inside."""
    x, y = np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)
    z = np.empty_like(y)
    z[0] = (y[1] - y[0]) / (x[1] - x[0])
    z[-1] = (y[-1] - y[-2]) / (x[-1] - x[-2])
    z[1:-1] = (y[2:] - y[:-2]) / (x[2:] - x[:-2])
    return z


def nedelec_splines(curve_B, curve_nu):
    """spl, spl_dnu of nedelec3D.jl:45-49: not-a-knot interpolating cubics (Dierckx
    Spline1D with s = 0), held at their end values outside the data (bc "nearest")."""
    from scipy.interpolate import CubicSpline
    x = np.asarray(curve_B, dtype=np.float64)
    s1 = CubicSpline(x, curve_nu, bc_type="not-a-knot")
    s2 = CubicSpline(x, fd_gradient(x, curve_nu), bc_type="not-a-knot")
    return (lambda b: s1(np.clip(b, x[0], x[-1]))), (lambda b: s2(np.clip(b, x[0], x[-1])))


def nedelec_newton(mesh, Bext, curve_B, curve_nu, nonlinear, nu_lin=None, tol=1e-4, max_newton=100, min_step=1e-4,
                   cg_rtol=1e-12):
    """Magnetostatics/nedelec3D.jl:149-231 with scipy's CG for the corrections."""
    import scipy.sparse.linalg as spla
    spl, spl_dnu = nedelec_splines(curve_B, curve_nu)
    nl = np.asarray(nonlinear, dtype=bool)
    nt = mesh.nt
    nu = np.ones(nt)
    if nu_lin is not None:
        nu[~nl] = np.asarray(nu_lin)[~nl]
    dnu = np.zeros(nt)
    rhs = nedelec_load(mesh, Bext)
    u = np.zeros(rhs.size)
    Bf, B = np.zeros((3, nt)), np.zeros(nt)
    att, div = 0, np.inf
    while div > tol and att < max_newton:
        att += 1
        Bold = B.copy()
        A = nedelecStiffness(mesh, nu)
        K = A + nedelecTangentialStiffness(mesh, dnu, Bf, B) if att > 1 else A
        du, _ = spla.cg(K, rhs - A @ u, rtol=cg_rtol, maxiter=100000)
        res_old = np.linalg.norm(rhs - A @ u)
        alf = 1.0
        trial = u + du
        res = np.linalg.norm(rhs - A @ trial)
        while res > res_old and alf > min_step:
            alf *= 0.9
            trial = u + alf * du
            res = np.linalg.norm(rhs - A @ trial)
        if not alf < min_step:
            u = trial
        Bf, B = nedelec_bfield(mesh, u)
        nu[nl] = spl(B[nl])
        dnu[nl] = spl_dnu(B[nl])
        div = np.abs(B - Bold).max()
    return u, Bf, B, nu, att


def quadraticStiffnessMatrix2D(mesh, mu=None, shift=True):
    """``src/FEM2D.jl:80-137``."""
    p, t = _pt(mesh)
    mv = None if mu is None else _c(mu, np.float64)
    return _assemble(lib().or_p2_stiffness2d, mesh, 6, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), _ptr(mv),
                     int(shift))


def quadraticMassMatrix2D(mesh):
    """``src/FEM2D.jl:163-229``."""
    p, t = _pt(mesh)
    return _assemble(lib().or_p2_mass2d, mesh, 6, p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64))


def lagrange(mesh):
    _, t = _pt(mesh)
    C_ = np.zeros(mesh.nv)
    lib().or_lagrange(t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), C_)
    return C_


def BoundaryIntegral(mesh, F, shell_id=(1,)):
    sT = _c(mesh.surfaceT.T, np.int32)
    RHS = np.zeros(mesh.nv)
    lib().or_boundary_integral(sT, mesh.ns, mesh.nv, _c(mesh.normal.T, np.float64), _c(mesh.AE, np.float64),
                               _c(F, np.float64), _c(shell_id, np.int32), len(shell_id), RHS)
    return RHS


def face_areas(mesh):
    """areaTriangle of the C++ reference (src/FEMc.cpp:44-53): |AB x AC| / 2 from p."""
    a, b, c = (mesh.p[:, mesh.surfaceT[q]] for q in range(3))
    return 0.5 * np.linalg.norm(np.cross((b - a).T, (c - a).T), axis=1)


def scalarPotential(mesh, mu, Hext, shell_id, tol=1e-13, maxit=1_000_000):
    """magnetostatics() of Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:5-38:
    RHS = BoundaryIntegral(p, surfaceT, normal, Hext, shell_id) with the face areas
    from p (src/FEMc.cpp:170-200), A = stiffnessMatrix(p, t, VE, mu) (:74-125), and
    u = A \\ (-RHS) by diagonal-preconditioned CG from u = 0 (Eigen's
    ConjugateGradient).  shell_id is the id as stored in surfaceT row 4.
    Returns (u, iterations, relres)."""
    sT = _c(mesh.surfaceT.T, np.int32)
    RHS = np.zeros(mesh.nv)
    lib().or_boundary_integral(sT, mesh.ns, mesh.nv, _c(mesh.normal.T, np.float64), _c(face_areas(mesh), np.float64),
                               _c(Hext, np.float64), _c([shell_id], np.int32), 1, RHS)
    A = stiffnessMatrix(mesh, mu)
    return pcg(A, -RHS, tol=tol, maxit=maxit)


def pcg(A, b, x0=None, fixed=None, tol=1e-10, maxit=100000):
    """Jacobi-PCG on a symmetric CSC matrix; returns (x, iterations, relres)."""
    A = sp.csc_matrix(A)
    n = A.shape[0]
    x = np.zeros(n) if x0 is None else _c(x0, np.float64).copy()
    fx = None if fixed is None else _c(fixed, np.uint8)
    rr = C.c_double()
    it = lib().or_pcg(n, _c(A.indptr, np.int64), _c(A.indices, np.int32), _c(A.data, np.float64),
                      _c(b, np.float64), x, _ptr(fx), tol, maxit, C.byref(rr))
    return x, it, rr.value


def hfield(mesh, u, ref_bug_hz=False):
    p, t = _pt(mesh)
    H = np.zeros(3 * mesh.nt)
    lib().or_hfield(p, t, mesh.nt, _c(u, np.float64), int(ref_bug_hz), H)
    return H.reshape(mesh.nt, 3).T


def froehlich(H, Ms, Hk):
    mu, dmu = C.c_double(), C.c_double()
    lib().or_froehlich(float(H), Ms, Hk, C.byref(mu), C.byref(dmu))
    return mu.value, dmu.value


def energy(mesh, H, nl, mu_lin, Ms=0.0, Hk=1.0):
    nlv = None if nl is None else _c(nl, np.uint8)
    return lib().or_energy(_c(np.asarray(H).T, np.float64), _c(mesh.VE, np.float64), mesh.nt, _ptr(nlv),
                           _c(mu_lin, np.float64), Ms, Hk)


LS_MODES = {"none": 0, "reference": 1, "residual": 2, "quadratic": 3}


def newton(mesh, u0, nl, mu_lin, Ms, Hk, tol_update=1e-8, maxit=100, cg_tol=1e-12, cg_maxit=200000,
           ref_bug_hz=False, line_search="residual", forcing="fixed", eta_min=1e-2, eta_max=0.3, picard_steps=0):
    """Dirichlet Newton-Raphson magnetostatics; returns (u, H 3 x nt, mu, stats dict).
    forcing="fixed" solves every increment to cg_tol; "ew" uses Eisenstat-Walker tolerances.
    picard_steps: first iterations with the secant operator only (no tangent term)."""
    p, t = _pt(mesh)
    u = _c(u0, np.float64).copy()
    H = np.zeros(3 * mesh.nt)
    mu = np.zeros(mesh.nt)
    st = np.zeros(6)
    lib().or_newton(p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), mesh.dirichlet_mask(), _c(nl, np.uint8),
                    _c(mu_lin, np.float64), Ms, Hk, tol_update, maxit, cg_tol, cg_maxit, int(ref_bug_hz),
                    LS_MODES[line_search], {"fixed": 0, "ew": 1}[forcing], eta_min, eta_max, int(picard_steps), u,
                    H, mu, st)
    stats = dict(newton_iters=int(st[0]), cg_iters=int(st[1]), update_ratio=st[2], residual=st[3], alpha=st[4],
                 converged=bool(st[5]))
    return u, H.reshape(mesh.nt, 3).T, mu, stats


def linear_magnetostatics(mesh, u0, mu, cg_tol=1e-10, cg_maxit=200000):
    p, t = _pt(mesh)
    u = _c(u0, np.float64).copy()
    H = np.zeros(3 * mesh.nt)
    it = C.c_int()
    lib().or_linear_magnetostatics(p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), mesh.dirichlet_mask(),
                                   _c(mu, np.float64), cg_tol, cg_maxit, u, H.ctypes.data_as(C.c_void_p), C.byref(it))
    return u, H.reshape(mesh.nt, 3).T, it.value


def heat_be(mesh, T0, kappa, rho_c, dt, nsteps, cg_tol=1e-10, cg_maxit=200000, every=10):
    p, t = _pt(mesh)
    T = _c(T0, np.float64).copy()
    nsnap = nsteps // every if every > 0 else 0
    snaps = np.zeros((max(nsnap, 1), mesh.nv))
    tot = C.c_int()
    lib().or_heat_be(p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), mesh.dirichlet_mask(), _c(kappa, np.float64),
                     rho_c, dt, nsteps, cg_tol, cg_maxit, T, every, snaps.ctypes.data_as(C.c_void_p), C.byref(tot))
    return T, snaps[:nsnap], tot.value


def objective_hx(mesh, target, u):
    p, t = _pt(mesh)
    return lib().or_objective_hx(p, t, mesh.nt, _c(mesh.VE, np.float64), _c(target, np.uint8), _c(u, np.float64))


def adjoint(mesh, target, mu, u, H=None, dmu=None, cg_tol=1e-12, cg_maxit=200000):
    """dJ/dmu per element (absolute permeability); returns (grad, lambda)."""
    p, t = _pt(mesh)
    lam = np.zeros(mesh.nv)
    grad = np.zeros(mesh.nt)
    Hc = None if H is None else _c(np.asarray(H).T, np.float64)
    dc = None if dmu is None else _c(dmu, np.float64)
    lib().or_adjoint(p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), mesh.dirichlet_mask(), _c(target, np.uint8),
                     _c(mu, np.float64), _ptr(Hc), _ptr(dc), _c(u, np.float64), cg_tol, cg_maxit, lam, grad)
    return grad, lam


def magnetostaticField(mesh, M, inside, cg_tol=1e-12, cg_maxit=200000):
    """Demagnetising field on the nodes (Micromagnetics/LL.jl:162-211); M is 3 x nv.
    Returns (Hn 3 x nv, u, CG iterations)."""
    p, t = _pt(mesh)
    u = np.zeros(mesh.nv)
    Hn = np.zeros(3 * mesh.nv)
    it = C.c_int()
    lib().or_demag_field(p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), _c(inside, np.uint8),
                         _c(np.asarray(M).T, np.float64), cg_tol, cg_maxit, u, Hn, C.byref(it))
    return Hn.reshape(mesh.nv, 3).T, u, it.value


def newton_sample(mesh, u, nl, mu_lin, Ms, Hk, cg_iters):
    """Times the pieces of one Newton iteration (seconds): state, tangent, cg_iters PCG iterations."""
    p, t = _pt(mesh)
    times = np.zeros(4)
    lib().or_newton_sample(p, t, mesh.nv, mesh.nt, _c(mesh.VE, np.float64), mesh.dirichlet_mask(), _c(nl, np.uint8),
                           _c(mu_lin, np.float64), Ms, Hk, _c(u, np.float64), int(cg_iters), times)
    return dict(state_s=times[0], tangent_s=times[1], cg_s=times[2], cg_iters=int(times[3]))
