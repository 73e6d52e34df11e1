"""Host-side mirror of Femeko's FEM hot-path interface on top of libfemeko_gpu.so.

Names, argument meaning and return types follow the reference functions, so a
script written against the reference reads the same:

==============================  =============================================  ==========================
this module                     reference (Femeko.jl)                          returns
==============================  =============================================  ==========================
stiffnessMatrix(mesh, f)        src/FEM3D.jl:40-56                             scipy CSC (SparseMatrixCSC)
localStiffnessMatrix(mesh, f)   src/FEM3D.jl:59-76                             (16, nt) ndarray
tangentialStiffnessMatrix       src/FEM3D.jl:79-119                            scipy CSC
massMatrix(mesh)                src/FEM3D.jl:466-492                           scipy CSC
stiffnessMatrix2D / massMatrix2D  src/FEM2D.jl:48-76, 139-161                  scipy CSC
quadraticStiffnessMatrix        src/FEM3D.jl:378-395                           scipy CSC
quadraticMassMatrix             src/FEM3D.jl:494-561                           scipy CSC
quadraticStiffnessMatrix2D      src/FEM2D.jl:117-137                           scipy CSC
quadraticMassMatrix2D           src/FEM2D.jl:163-229                           scipy CSC
lagrange(mesh)                  src/FEM3D.jl:274-281                           ndarray (nv)
BoundaryIntegral(mesh, F)       src/FEM3D.jl:284-297                           ndarray (nv)
cg(A, b)                        IterativeSolvers.cg (e.g. run.jl:141)          ndarray
magnetostatics_linear           Magnetostatics/magneticField.jl:89-132         (u, H, stats)
newton_magnetostatics           Magnetostatics/NewtonRaphson.jl:109-214        (u, H, mu, stats)
hfield(mesh, u)                 Magnetostatics/magneticField.jl:111-124        (3, nt) ndarray
heat_be                         Heat/heat3D.jl:50-90                           (T, snapshots, stats)
magnetostaticField              Micromagnetics/LL.jl:162-211                   (Hn 3 x nv, u, stats)
batch_magnetostatics_linear     magneticField.jl:89-132 on many meshes         (u list, iters, stats)
magnetostatics_sweep            magneticField.jl:89-132 for many fields        (U nv x nfield, stats)
adjoint_dJdmu                   (none: gradient of NewtonRaphson.jl:234-240)   (J, grad, u, stats)
==============================  =============================================  ==========================

The mesh argument is a :class:`femeko_gpu.mesh.MESH` (the reference struct's fields).
The first GPU call on a mesh uploads it and builds the sparse pattern once; the
device handle is cached on the mesh object.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import _lib as L
from .mesh import MESH, MU0, box_tet_mesh, box_tri_mesh, surface_faces6, surface_lines3, surface_faces_p2  # noqa: F401
from .meshio import load_mesh, save_mesh, save2file, load2array  # noqa: F401

__all__ = [
    "GPUMesh", "gpu_mesh", "lagrange", "BoundaryIntegral", "stiffnessMatrix", "localStiffnessMatrix", "tangentialStiffnessMatrix", "quadraticConvectionMatrix", "quadraticBoundaryMassMatrix", "transport_be", "surface_faces6", "massMatrix",
    "stiffnessMatrix2D", "massMatrix2D", "quadraticStiffnessMatrix", "quadraticMassMatrix",
    "quadraticStiffnessMatrix2D", "quadraticMassMatrix2D", "cg", "spmv", "magnetostatics_linear",
    "newton_magnetostatics", "ResidentNewton", "hfield", "heat_be", "adjoint_dJdmu", "magnetostaticField", "batch_magnetostatics_linear", "magnetostatics_sweep", "solve_opts", "newton_opts", "MESH", "MU0", "box_tet_mesh", "box_tri_mesh",
    "load_mesh", "save_mesh", "save2file", "load2array",
]


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class GPUMesh:
    """Owns one fg_mesh handle: the mesh, its pattern and its work buffers on the GPU."""

    def __init__(self, mesh: MESH, dirichlet: bool = True):
        lib = L.lib()
        self.mesh = mesh
        self._p = _c(mesh.p.T, np.float64)          # 3 x nv column-major
        self._t = _c(mesh.t.T, np.int32)            # npe x nt column-major
        h = C.c_void_p()
        L.check(lib.fg_mesh_create(L.ptr(self._p), mesh.nv, L.ptr(self._t), mesh.nt, mesh.npe, 0, C.byref(h)))
        self.h = h
        L.register_handle(self)
        nnz, mr = C.c_int64(), C.c_int32()
        L.check(lib.fg_mesh_nnz(h, C.byref(nnz), C.byref(mr)))
        self.nnz, self.max_row = nnz.value, mr.value
        colptr = np.zeros(mesh.nv + 1, dtype=np.int64)
        rowval = np.zeros(self.nnz, dtype=np.int32)
        L.check(lib.fg_csc_pattern(h, L.ptr(colptr), L.ptr(rowval), 0))
        self.colptr, self.rowval = colptr, rowval
        if dirichlet and mesh.boundary_nodes is not None:
            self.set_dirichlet(mesh.dirichlet_mask())

    def set_dirichlet(self, fixed):
        f = None if fixed is None else _c(fixed, np.uint8)
        L.check(L.lib().fg_mesh_set_dirichlet(self.h, L.ptr(f)))

    def volumes(self):
        VE = np.zeros(self.mesh.nt)
        L.check(L.lib().fg_mesh_volumes(self.h, L.ptr(VE)))
        return VE

    def csc(self, vals):
        n = self.mesh.nv
        return sp.csc_matrix((vals, self.rowval.copy(), self.colptr.copy()), shape=(n, n))

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


def gpu_mesh(mesh: MESH) -> GPUMesh:
    g = getattr(mesh, "_gpu", None)
    if g is None or g.h is None:
        g = GPUMesh(mesh)
        object.__setattr__(mesh, "_gpu", g)
    return g


def _assemble(mesh, fn, *args):
    g = gpu_mesh(mesh)
    vals = np.zeros(g.nnz)
    L.check(fn(g.h, *args, L.ptr(vals)))
    return g.csc(vals)


def stiffnessMatrix(mesh: MESH, f=None):
    """Global stiffness matrix; P1/P2, tetrahedra or triangles by ``mesh.t``'s rows."""
    fv = None if f is None else _c(f, np.float64)
    return _assemble(mesh, L.lib().fg_stiffness, L.ptr(fv))


stiffnessMatrix2D = stiffnessMatrix
quadraticStiffnessMatrix = stiffnessMatrix
quadraticStiffnessMatrix2D = stiffnessMatrix


def massMatrix(mesh: MESH, F=None, full_phi: bool = False):
    """Global mass matrix.  For P2 tetrahedra ``full_phi=False`` reproduces the
    reference's linear-part-only basis evaluation (src/FEM3D.jl:529-531)."""
    fv = None if F is None else _c(F, np.float64)
    return _assemble(mesh, L.lib().fg_mass, L.ptr(fv), int(full_phi))


massMatrix2D = massMatrix
quadraticMassMatrix = massMatrix
quadraticMassMatrix2D = massMatrix


def quadraticConvectionMatrix(mesh: MESH, u, F=None, full_phi: bool = False):
    """Global P2 convection matrix of the nodal velocity ``u`` (3 x nv), as
    src/FEM3D.jl:563-648 builds it for tetrahedra (entry (t_i, t_j) sums the local
    Ck[j, i]; ``full_phi=False`` keeps the reference's linear-part-only phi) and
    src/FEM2D.jl:231-319 for triangles (u interpolated with the P2 basis; F should be
    None: the 2D reference has no factor)."""
    uv = _c(np.asarray(u, dtype=np.float64).T, np.float64)   # 3 x nv column-major
    fv = None if F is None else _c(F, np.float64)
    return _assemble(mesh, L.lib().fg_convection, L.ptr(uv), L.ptr(fv), int(full_phi))


def tangentialStiffnessMatrix(mesh: MESH, H_vec, dmu):
    H = _c(np.asarray(H_vec, dtype=np.float64).T, np.float64)   # 3 x nt column-major
    d = _c(dmu, np.float64)
    return _assemble(mesh, L.lib().fg_tangent, L.ptr(H), L.ptr(d))


def localStiffnessMatrix(mesh: MESH, f=None):
    g = gpu_mesh(mesh)
    fv = None if f is None else _c(f, np.float64)
    Ak = np.zeros(16 * mesh.nt)
    L.check(L.lib().fg_local_stiffness(g.h, L.ptr(fv), L.ptr(Ak)))
    return Ak.reshape(mesh.nt, 16).T


def lagrange(mesh: MESH):
    """Lagrange-multiplier row C_i = sum over the elements of node i of VE/4 (src/FEM3D.jl:274-281)."""
    g = gpu_mesh(mesh)
    C_ = np.zeros(mesh.nv)
    L.check(L.lib().fg_lagrange(g.h, L.ptr(C_)))
    return C_


def BoundaryIntegral(mesh: MESH, F, shell_id=(1,)):
    """Neumann right-hand side (n . F) AE / 3 on the faces of the given boundary ids (src/FEM3D.jl:284-297)."""
    g = gpu_mesh(mesh)
    sT = _c(mesh.surfaceT.T, np.int32)
    RHS = np.zeros(mesh.nv)
    sh = _c(shell_id, np.int32)
    L.check(L.lib().fg_boundary_integral(g.h, L.ptr(sT), mesh.ns, 0, L.ptr(_c(mesh.normal.T, np.float64)),
                                         L.ptr(_c(mesh.AE, np.float64)), L.ptr(_c(F, np.float64)), L.ptr(sh),
                                         len(sh), L.ptr(RHS)))
    return RHS


def solve_opts(precision="fp64", rtol=1e-10, maxiter=1_000_000, inner_rtol=1e-5, check_every=32, use_graph=True,
               spmv=0):
    """Linear-solve options; spmv = 0 autotunes the FP32 CG iteration kernel, 1..29 forces a variant."""
    o = L.SolveOpts()
    L.lib().fg_solve_opts_default(C.byref(o))
    o.precision = L.FG_MIXED if precision == "mixed" else L.FG_FP64
    o.rtol, o.maxiter, o.inner_rtol = rtol, maxiter, inner_rtol
    o.check_every, o.use_graph, o.spmv = check_every, int(use_graph), int(spmv)
    return o


def newton_opts(precision="mixed", tol_update=1e-8, maxit=100, inner_rtol=1e-4, cg_maxiter=200_000,
                line_search="residual", min_step=1e-4, Ms=1.2e6, Hk=500.0, check_every=32, use_graph=True,
                forcing="ew", eta_min=1e-2, eta_max=0.3, picard_steps=2):
    """Newton options.  forcing="ew": Eisenstat-Walker inner tolerances in
    [eta_min, eta_max]; forcing="fixed": every inner solve to inner_rtol.
    picard_steps: first iterations without the tangent term."""
    o = L.NewtonOpts()
    L.lib().fg_newton_opts_default(C.byref(o))
    o.forcing = {"fixed": 0, "ew": 1}[forcing]
    o.picard_steps = int(picard_steps)
    o.eta_min, o.eta_max = eta_min, eta_max
    o.precision = L.FG_MIXED if precision == "mixed" else L.FG_FP64
    o.tol_update, o.maxit, o.inner_rtol, o.cg_maxiter = tol_update, maxit, inner_rtol, cg_maxiter
    o.line_search = {"none": L.FG_LS_NONE, "reference": L.FG_LS_REFERENCE, "residual": L.FG_LS_RESIDUAL,
                     "quadratic": L.FG_LS_QUADRATIC}[line_search]
    o.min_step, o.Ms, o.Hk, o.check_every, o.use_graph = min_step, Ms, Hk, check_every, int(use_graph)   # 2: host-checked blocks
    return o


def cg(A, b, x0=None, reltol=1e-10, maxiter=1_000_000, precision="fp64", return_stats=False, **kw):
    """Jacobi-preconditioned CG on a symmetric sparse matrix (IterativeSolvers.cg drop-in)."""
    A = sp.csc_matrix(A)
    n = A.shape[0]
    colptr = _c(A.indptr, np.int64)
    rowval = _c(A.indices, np.int64)
    nz = _c(A.data, np.float64)
    x = np.zeros(n) if x0 is None else _c(x0, np.float64).copy()
    o = solve_opts(precision=precision, rtol=reltol, maxiter=maxiter, **kw)
    s = L.SolveStats()
    st = L.lib().fg_cg_csc(n, L.ptr(colptr), L.ptr(rowval), L.ptr(nz), 0, L.ptr(_c(b, np.float64)), L.ptr(x),
                           C.byref(o), C.byref(s))
    L.check(st, allow_not_converged=True)
    return (x, L.stats_dict(s)) if return_stats else x


def spmv(A, x):
    A = sp.csc_matrix(A)
    n = A.shape[0]
    y = np.zeros(n)
    L.check(L.lib().fg_spmv_csc(n, L.ptr(_c(A.indptr, np.int64)), L.ptr(_c(A.indices, np.int64)),
                                L.ptr(_c(A.data, np.float64)), 0, L.ptr(_c(x, np.float64)), L.ptr(y)))
    return y


def magnetostatics_linear(mesh: MESH, mu, u_in, precision="fp64", rtol=1e-10, **kw):
    """K(mu) u = 0 on interior rows with u = u_in on the Dirichlet rows."""
    g = gpu_mesh(mesh)
    u = np.zeros(mesh.nv)
    H = np.zeros(3 * mesh.nt)
    o = solve_opts(precision=precision, rtol=rtol, **kw)
    s = L.SolveStats()
    st = L.lib().fg_magnetostatics_linear(g.h, L.ptr(_c(mu, np.float64)), L.ptr(_c(u_in, np.float64)), C.byref(o),
                                          L.ptr(u), L.ptr(H), C.byref(s))
    L.check(st, allow_not_converged=True)
    return u, H.reshape(mesh.nt, 3).T, L.stats_dict(s)


def scalarPotential(mesh: MESH, mu, Hext, shell_id, precision="mixed", rtol=1e-12, reference_call=False, **kw):
    """Linear Neumann magnetostatics of the C++ reference's ``scalarPotential``
    (Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:5-95): u with
    K(mu) u = -BoundaryIntegral(Hext) over the faces whose id equals ``shell_id``
    (ids as stored in ``mesh.surfaceT`` row 4), solved from u = 0 by Jacobi-PCG.
    reference_call=True goes through the void ``scalarPotential`` symbol with the
    reference's 0-based argument layout (Femeko_jl_C++/Magnetostatics/run.jl:49-79);
    otherwise through ``fg_scalar_potential`` with options.  Returns (u, stats)."""
    # the reference's layout (run.jl:49-52): 0-based nodes, and the boundary ids and
    # shell id shifted down by one alongside them; this mesh holds 0-based nodes and
    # the reference's 1-based ids
    # (column-major 3 x nv, 4 x nt, 4 x ns, 3 x ns: C order of the transposes)
    t0 = _c(mesh.t.T, np.int32)
    sT = np.array(mesh.surfaceT, dtype=np.int32, copy=True)
    sT[3] -= 1
    sT = _c(sT.T, np.int32)
    shell = int(shell_id) - 1
    p = _c(mesh.p.T, np.float64)
    nrm = _c(mesh.normal.T, np.float64)
    VE = _c(mesh.VE, np.float64)
    muv = _c(mu, np.float64)
    H = _c(Hext, np.float64)
    u = np.zeros(mesh.nv)
    lib = L.lib()
    args = (L.ptr(u), L.ptr(p), L.ptr(t0), L.ptr(sT), L.ptr(nrm), int(mesh.nv), int(mesh.nt),
            int(sT.shape[0]), L.ptr(VE), L.ptr(muv), L.ptr(H), shell)
    if reference_call:
        lib.scalarPotential(*args)
        st = lib.fg_scalar_potential_status()
        L.check(st, allow_not_converged=True)
        return u, {"status": st}
    o = solve_opts(precision=precision, rtol=rtol, **kw)
    s = L.SolveStats()
    L.check(lib.fg_scalar_potential(*args, C.byref(o), C.byref(s)), allow_not_converged=True)
    return u, L.stats_dict(s)


def newton_magnetostatics(mesh: MESH, nl, mu_lin, u0, **kw):
    """Nonlinear Newton-Raphson magnetostatics; returns (u, H, mu, stats)."""
    g = gpu_mesh(mesh)
    u = np.zeros(mesh.nv)
    H = np.zeros(3 * mesh.nt)
    mu = np.zeros(mesh.nt)
    o = newton_opts(**kw)
    s = L.NewtonStats()
    st = L.lib().fg_newton_magnetostatics(g.h, L.ptr(_c(nl, np.uint8)), L.ptr(_c(mu_lin, np.float64)),
                                          L.ptr(_c(u0, np.float64)), C.byref(o), L.ptr(u), L.ptr(H), L.ptr(mu),
                                          C.byref(s))
    L.check(st, allow_not_converged=True)
    return u, H.reshape(mesh.nt, 3).T, mu, L.stats_dict(s)


def heat_be(mesh: MESH, T0, kappa, rho_c=1.0, dt=1e-3, nsteps=100, every=10, precision="fp64", rtol=1e-10,
            check_every=8, **kw):
    """Backward-Euler heat steps (Heat/heat3D.jl:50-90) with T = 0 on the Dirichlet
    nodes; returns (T_final, snapshots every `every` steps, stats).  Each step's solve
    takes a few tens of CG iterations, so its graph loop tests for convergence every
    `check_every` = 8 iterations (fewer idle launches after convergence)."""
    g = gpu_mesh(mesh)
    T = _c(T0, np.float64).copy()
    nsnap = nsteps // every if every > 0 else 0
    snaps = np.zeros((max(nsnap, 1), mesh.nv))
    o = solve_opts(precision=precision, rtol=rtol, check_every=check_every, **kw)
    s = L.SolveStats()
    st = L.lib().fg_heat_be(g.h, L.ptr(_c(kappa, np.float64)), rho_c, dt, nsteps, L.ptr(T), every,
                            L.ptr(snaps) if nsnap else None, C.byref(o), C.byref(s))
    L.check(st, allow_not_converged=True)
    return T, snaps[:nsnap], L.stats_dict(s)


def quadraticBoundaryMassMatrix(mesh: MESH, F=None, faces=None):
    """P2 boundary mass with the per-face factor F (ns, default ones): surface
    triangles of a tetrahedral mesh (src/FEM3D.jl:300-322, ``faces`` 6 x ns) or
    boundary lines of a triangle mesh (quadraticMassMatrix1D, src/FEM2D.jl:394-419,
    ``faces`` 3 x ns); ``faces`` defaults to ``surface_faces_p2(mesh)``."""
    g = gpu_mesh(mesh)
    f6 = surface_faces_p2(mesh) if faces is None else np.asarray(faces)
    ns = f6.shape[1]
    vals = np.zeros(g.nnz)
    Fv = None if F is None else _c(F, np.float64)
    L.check(L.lib().fg_boundary_mass(g.h, L.ptr(_c(f6.T, np.int32)), L.ptr(_c(mesh.AE[:ns], np.float64)),
                                     L.ptr(Fv), ns, L.ptr(vals)))
    return g.csc(vals)


quadraticMassMatrix1D = quadraticBoundaryMassMatrix
quadraticConvectionMatrix2D = quadraticConvectionMatrix


def transport_be(mesh: MESH, T0, rho_cp, kappa, u, dt, nsteps, face_F=None, faces=None, full_phi=True, every=0,
                 rtol=1e-10, maxiter=10_000):
    """Backward-Euler transport steps T <- LM \\ (M T), LM = M + dt (A + R + C)
    (Transport/main3D.jl:143-213) with Jacobi-BiCGStab on the GPU.  u: 3 x nv velocity;
    face_F: per-surface-face penalty factor (the reference's intakeBC; None = no R).
    Returns (T_final, snapshots every `every` steps, stats with "status" 0/1/2)."""
    g = gpu_mesh(mesh)
    T = _c(T0, np.float64).copy()
    nsnap = nsteps // every if every > 0 else 0
    snaps = np.zeros((max(nsnap, 1), mesh.nv))
    if face_F is None:
        f6, AE, Fv, nf = None, None, None, 0
    else:
        f6 = _c((surface_faces_p2(mesh) if faces is None else np.asarray(faces)).T, np.int32)
        nf = f6.shape[0]
        AE, Fv = _c(mesh.AE[:nf], np.float64), _c(face_F, np.float64)
    uv = _c(np.asarray(u, dtype=np.float64).T, np.float64)
    o = solve_opts(precision="fp64", rtol=rtol, maxiter=maxiter)
    s = L.SolveStats()
    st = L.lib().fg_transport_be(g.h, L.ptr(_c(rho_cp, np.float64)), L.ptr(_c(kappa, np.float64)), L.ptr(uv),
                                 L.ptr(f6), L.ptr(AE), L.ptr(Fv), nf, float(dt), int(nsteps), int(full_phi),
                                 L.ptr(T), every, L.ptr(snaps) if nsnap else None, C.byref(o), C.byref(s))
    L.check(st, allow_not_converged=True)
    d = L.stats_dict(s)
    d["status"] = s.pad_
    return T, snaps[:nsnap], d


def magnetostatics_sweep(mesh: MESH, mu, H0, rtol=1e-10, inner_rtol=1e-5, maxiter=1_000_000, check_every=16,
                         method="block"):
    """Linear magnetostatics for many applied fields H0 (nfield x 3) at once, FP32
    inner iterations + FP64 refinement; returns (U nv x nfield, stats).
    method="block": the fields' rank-revealing reduction to r <= 3 field directions
    and one block CG of width r (stats["rank"] = r); "per_field": one CG per field
    sharing every matrix read."""
    g = gpu_mesh(mesh)
    H = _c(np.asarray(H0, dtype=np.float64).reshape(-1, 3), np.float64)   # 3 x nfield column-major
    nf = H.shape[0]
    U = np.zeros((nf, mesh.nv))                                             # column-major nv x nf
    o = solve_opts(precision="mixed", rtol=rtol, inner_rtol=inner_rtol, maxiter=maxiter, check_every=check_every,
                   spmv={"block": 0, "per_field": 1}[method])
    s = L.SolveStats()
    st = L.lib().fg_magnetostatics_sweep(g.h, L.ptr(_c(mu, np.float64)), nf, L.ptr(H), C.byref(o), L.ptr(U),
                                         C.byref(s))
    L.check(st, allow_not_converged=True)
    d = L.stats_dict(s)
    if method == "block":
        d["rank"] = s.pad_
    return U.T, d


def batch_magnetostatics_linear(meshes, mus, u_ins, rtol=1e-10, maxiter=1_000_000, precision="fp64",
                                inner_rtol=1e-5):
    """Independent linear magnetostatic problems (one per mesh, Dirichlet rows from
    each mesh) in one persistent GPU launch; returns (list of u, iterations, stats).
    precision "mixed" runs FP32 PCG inside FP64 refinement on each problem's cluster
    (iterations are then the inner FP32 iterations)."""
    gs = [gpu_mesh(m) for m in meshes]
    n = len(meshes)
    mus_c = [_c(mu, np.float64) for mu in mus]
    uin_c = [_c(u, np.float64) for u in u_ins]
    outs = [np.zeros(m.nv) for m in meshes]
    H = (C.c_void_p * n)(*[g.h.value for g in gs])
    MU = (C.c_void_p * n)(*[a.ctypes.data for a in mus_c])
    UI = (C.c_void_p * n)(*[a.ctypes.data for a in uin_c])
    UO = (C.c_void_p * n)(*[a.ctypes.data for a in outs])
    its = np.zeros(n, dtype=np.int32)
    o = solve_opts(precision=precision, rtol=rtol, maxiter=maxiter, inner_rtol=inner_rtol)
    s = L.BatchStats()
    st = L.lib().fg_batch_magnetostatics_linear(H, n, MU, UI, C.byref(o), UO, L.ptr(its), C.byref(s))
    L.check(st, allow_not_converged=True)
    return outs, its, L.stats_dict(s)


def adjoint_dJdmu(mesh: MESH, mur, u0, target, nl=None, rtol=1e-12, **kw):
    """J = volume-weighted mean Hx over the target elements and dJ/dmur per element
    through the GPU adjoint; nl = None solves the linear problem, else the Newton one.
    Returns (J, grad, u, stats)."""
    g = gpu_mesh(mesh)
    grad = np.zeros(mesh.nt)
    u = np.zeros(mesh.nv)
    J = C.c_double()
    o = newton_opts(**kw)
    s = L.AdjointStats()
    nlp = None if nl is None else L.ptr(_c(nl, np.uint8))
    st = L.lib().fg_adjoint_dJdmu(g.h, L.ptr(_c(mur, np.float64)), L.ptr(_c(u0, np.float64)),
                                  L.ptr(_c(target, np.uint8)), nlp, C.byref(o), rtol, C.byref(J), L.ptr(grad),
                                  L.ptr(u), C.byref(s))
    L.check(st, allow_not_converged=True)
    return J.value, grad, u, L.stats_dict(s)


def magnetostaticField(mesh: MESH, M, inside, precision="fp64", rtol=1e-10, **kw):
    """Demagnetising field on the nodes (Micromagnetics/LL.jl:162-211); M is 3 x nv,
    inside the nt mask of the magnetic body.  Like the reference, the Poisson problem
    has no Dirichlet rows.
    Returns (Hn 3 x nv, u, stats)."""
    # a handle of its own without Dirichlet rows, kept on the mesh so that the
    # operator stays assembled from one micromagnetic step to the next
    g = getattr(mesh, "_gpu_demag", None)
    if g is None or g.h is None:
        g = GPUMesh(mesh, dirichlet=False)
        object.__setattr__(mesh, "_gpu_demag", g)
    Hn = np.zeros(3 * mesh.nv)
    u = np.zeros(mesh.nv)
    o = solve_opts(precision=precision, rtol=rtol, **kw)
    s = L.SolveStats()
    st = L.lib().fg_demag_field(g.h, L.ptr(_c(inside, np.uint8)), L.ptr(_c(np.asarray(M).T, np.float64)),
                                C.byref(o), L.ptr(Hn), L.ptr(u), C.byref(s))
    L.check(st, allow_not_converged=True)
    return Hn.reshape(mesh.nv, 3).T, u, L.stats_dict(s)


class ResidentNewton:
    """Newton magnetostatics kept on the device: inputs uploaded once, each solve()
    runs from them and leaves u, H, mu on the GPU until outputs() downloads them."""

    def __init__(self, mesh: MESH, nl, mu_lin, u0):
        self.mesh = mesh
        self.g = gpu_mesh(mesh)
        self._in = (_c(nl, np.uint8), _c(mu_lin, np.float64), _c(u0, np.float64))
        L.check(L.lib().fg_newton_set_inputs(self.g.h, *(L.ptr(a) for a in self._in)))

    def solve(self, **kw):
        o = newton_opts(**kw)
        s = L.NewtonStats()
        L.check(L.lib().fg_newton_solve_resident(self.g.h, C.byref(o), C.byref(s)), allow_not_converged=True)
        return L.stats_dict(s)

    def outputs(self):
        m = self.mesh
        u, H, mu = np.zeros(m.nv), np.zeros(3 * m.nt), np.zeros(m.nt)
        L.check(L.lib().fg_newton_get_outputs(self.g.h, L.ptr(u), L.ptr(H), L.ptr(mu)))
        return u, H.reshape(m.nt, 3).T, mu


def hfield(mesh: MESH, u):
    g = gpu_mesh(mesh)
    H = np.zeros(3 * mesh.nt)
    L.check(L.lib().fg_hfield(g.h, L.ptr(_c(u, np.float64)), L.ptr(H)))
    return H.reshape(mesh.nt, 3).T


from .nedelec import (edge_mesh, nedelec_edges, nedelecLocalStiffness, nedelecStiffness,  # noqa: E402,F401
                      nedelecTangentialStiffness, nedelec_load, nedelec_bfield, nedelec_linear, nedelec_newton)
