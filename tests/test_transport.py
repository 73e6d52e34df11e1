"""P2 transport (Transport/main3D.jl:143-213): convection, boundary mass and the
backward-Euler steps LM T_{n+1} = M T_n with LM = M + dt (A + R + C).  The oracle
builds the same matrices in C/numpy and solves each step directly (sparse LU), as the
reference's `\\` does; the GPU path iterates (Jacobi-BiCGStab) to a tight tolerance."""
import numpy as np
import pytest

import femeko_gpu as fg
from femeko_gpu.mesh import box_tet_mesh, surface_faces6
import oracle as O


def intake(m, x=-5.0):
    """Penalty factor 1e6 on the surface faces lying in the plane x = x (main3D.jl:143-151)."""
    f6 = surface_faces6(m)
    on = np.all(np.isclose(m.p[0][f6[:3]], x), axis=0)
    return f6, np.where(on, 1e6, 0.0)


def problem(n=3, seed=2):
    m = box_tet_mesh(n, seed=seed, order=2)
    rng = np.random.default_rng(seed)
    u = np.vstack([np.full(m.nv, 1.0), 0.3 * np.sin(m.p[2]), 0.1 * rng.normal(size=m.nv)])
    rho = rng.uniform(0.8, 1.2, m.nt)
    kap = rng.uniform(0.02, 0.08, m.nt)
    T0 = np.exp(-(m.p[0] ** 2 + m.p[1] ** 2) / 4)
    return m, u, rho, kap, T0


def test_surface_faces6_midpoints():
    m = box_tet_mesh(2, seed=1, order=2)
    f6 = surface_faces6(m)
    for r, (i, j) in enumerate(((0, 1), (1, 2), (2, 0))):
        assert np.allclose(m.p[:, f6[3 + r]], 0.5 * (m.p[:, f6[i]] + m.p[:, f6[j]]))


def test_boundary_mass_known_answers():
    """The P2 triangle basis sums to 1, so R sums to sum(AE F) and 1^T R T = int T dA
    (exact for T linear: the face centroid value times the area)."""
    m, _, _, _, _ = problem()
    f6, F = intake(m)
    R = O.quadraticBoundaryMassMatrix(m, f6, F)
    assert abs(R.sum() - (m.AE * F).sum()) <= 1e-12 * (m.AE * F).sum()
    a = np.array([0.5, -2.0, 1.0])
    T = a @ m.p
    cen = np.mean(m.p[:, f6[:3]], axis=1)                     # 3 x ns face centroids
    ref = np.sum(m.AE * F * (a @ cen))
    assert abs(np.ones(m.nv) @ (R @ T) - ref) <= 1e-10 * np.abs(m.AE * F).sum()
    assert abs(R - R.T).max() == 0.0


def test_transport_oracle_identity_step():
    """kappa = 0, u = 0 and no intake: LM = M, so a step returns T unchanged."""
    m, _, rho, _, T0 = problem(n=2)
    out = O.transport_be(m, T0, rho, np.zeros(m.nt), np.zeros((3, m.nv)), 0.1, 1)
    assert np.abs(out[0] - T0).max() < 1e-11


@pytest.mark.gpu
def test_boundary_mass_parity():
    m, _, _, _, _ = problem()
    f6, F = intake(m)
    Rg = fg.quadraticBoundaryMassMatrix(m, F, faces=f6)
    Ro = O.quadraticBoundaryMassMatrix(m, f6, F)
    D = (Rg - Ro).tocsc()
    assert abs(D).max() <= 1e-13 * abs(Ro).max()
    bad = f6.copy()
    bad[0, np.argmax(F)] = bad[0, np.argmin(F)] if F.min() == 0 else 0
    bad[1, np.argmax(F)] = m.nv - 1
    with pytest.raises(RuntimeError):
        fg.quadraticBoundaryMassMatrix(m, F, faces=bad)


@pytest.mark.gpu
@pytest.mark.parametrize("with_intake", [False, True])
def test_transport_parity(with_intake):
    m, u, rho, kap, T0 = problem()
    f6, F = intake(m) if with_intake else (None, None)
    dt, nsteps = 0.05, 4
    T, snaps, st = fg.transport_be(m, T0, rho, kap, u, dt, nsteps, face_F=F, faces=f6, every=2, rtol=1e-13)
    ref = O.transport_be(m, T0, rho, kap, u, dt, nsteps, f6, F)
    assert st["converged"] and st["status"] == 0 and st["iterations"] > 0
    scale = np.abs(ref[-1]).max()
    assert np.abs(T - ref[-1]).max() <= 1e-9 * scale
    assert np.abs(snaps[0] - ref[1]).max() <= 1e-9 * scale and np.abs(snaps[1] - T).max() == 0.0


@pytest.mark.gpu
def test_transport_repeatable_and_limits():
    m, u, rho, kap, T0 = problem(n=2)
    a = fg.transport_be(m, T0, rho, kap, u, 0.05, 2, rtol=1e-12)[0]
    b = fg.transport_be(m, T0, rho, kap, u, 0.05, 2, rtol=1e-12)[0]
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    # an iteration cap too small to converge is reported, not hidden
    _, _, st = fg.transport_be(m, T0, rho, kap, u, 0.05, 1, rtol=1e-14, maxiter=1)
    assert not st["converged"] and st["status"] == 1
    with pytest.raises(RuntimeError):     # P1 mesh
        pm = fg.box_tet_mesh(2, seed=1)
        fg.transport_be(pm, np.zeros(pm.nv), np.ones(pm.nt), np.ones(pm.nt), np.zeros((3, pm.nv)), 0.1, 1)


# ---------------------------------------------------------------- 2D (Transport/main2D.jl)
def problem2d(n=4, seed=3):
    m = fg.box_tri_mesh(n, seed=seed, order=2)
    rng = np.random.default_rng(seed)
    u = np.vstack([np.full(m.nv, 1.0), 0.3 * np.sin(m.p[0]), np.zeros(m.nv)])
    kap = rng.uniform(0.02, 0.08, m.nt)
    T0 = np.exp(-(m.p[0] ** 2 + m.p[1] ** 2) / 4)
    return m, u, kap, T0


def intake2d(m):
    from femeko_gpu.mesh import surface_lines3
    f3 = surface_lines3(m)
    xmin = m.p[0].min()
    on = np.all(np.isclose(m.p[0][f3[:2]], xmin), axis=0)
    return f3, np.where(on, 1e6, 0.0)


def test_convection2d_known_answers():
    """2D C[r, c] = int phi_r (u . grad phi_c) (src/FEM2D.jl:231-319 after its scatter):
    rows sum to 0 and, for constant u and linear T = a . x, C T = (u . a) M 1."""
    m, _, _, _ = problem2d()
    uc = np.vstack([np.full(m.nv, 0.7), np.full(m.nv, -0.4), np.zeros(m.nv)])
    C = O.quadraticConvectionMatrix2D(m, uc)
    a = np.array([1.5, -2.0])
    T = a @ m.p[:2]
    rhs = (np.array([0.7, -0.4]) @ a) * (O.quadraticMassMatrix2D(m) @ np.ones(m.nv))
    assert np.abs(C @ T - rhs).max() <= 1e-12 * np.abs(rhs).max()
    assert np.abs(np.asarray(C.sum(axis=1))).max() <= 1e-12 * np.abs(C.data).max()
    f3, F = intake2d(m)
    R = O.quadraticMassMatrix1D(m, f3, F)
    assert abs(R.sum() - (m.AE * F).sum()) <= 1e-12 * (m.AE * F).sum()


@pytest.mark.gpu
def test_transport2d_parity():
    m, u, kap, T0 = problem2d()
    Cg, Co = fg.quadraticConvectionMatrix(m, u), O.quadraticConvectionMatrix2D(m, u)
    assert np.array_equal(Cg.indptr, Co.indptr) and np.array_equal(Cg.indices, Co.indices)
    assert np.abs(Cg.data - Co.data).max() <= 1e-11 * np.abs(Co.data).max()
    f3, F = intake2d(m)
    Rg, Ro = fg.quadraticBoundaryMassMatrix(m, F, faces=f3), O.quadraticMassMatrix1D(m, f3, F)
    assert abs(Rg - Ro).max() <= 1e-13 * abs(Ro).max()
    ones = np.ones(m.nt)
    T, _, st = fg.transport_be(m, T0, ones, kap, u, 0.05, 4, face_F=F, faces=f3, rtol=1e-13)
    ref = O.transport_be(m, T0, ones, kap, u, 0.05, 4, f3, F)
    assert st["converged"]
    assert np.abs(T - ref[-1]).max() <= 1e-9 * np.abs(ref[-1]).max()


@pytest.mark.gpu
def test_transport_edge_cases():
    """Zero steps return T unchanged; faces whose factor is 0 change nothing (bit for
    bit); a face list given with no nonzero factor equals no faces at all."""
    m, u, rho, kap, T0 = problem(n=2)
    T, snaps, st = fg.transport_be(m, T0, rho, kap, u, 0.05, 0)
    assert np.array_equal(T, T0) and st["iterations"] == 0 and snaps.shape[0] == 0
    f6, F = intake(m)
    a = fg.transport_be(m, T0, rho, kap, u, 0.05, 2, rtol=1e-12)[0]
    b = fg.transport_be(m, T0, rho, kap, u, 0.05, 2, face_F=np.zeros_like(F), faces=f6, rtol=1e-12)[0]
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    c = fg.transport_be(m, T0, rho, kap, u, 0.05, 2, face_F=F, faces=f6, rtol=1e-12)[0]
    assert np.abs(c - a).max() > 0.0          # the intake penalty acts
    bad = f6.copy()
    bad[0, 0] = bad[1, 0]                     # a face repeating a node
    with pytest.raises(RuntimeError):
        fg.transport_be(m, T0, rho, kap, u, 0.05, 1, face_F=np.ones_like(F), faces=bad)
