"""Nedelec edge elements (src/FEM3D.jl:155-271, Magnetostatics/nedelec3D.jl:106-221):
GPU element blocks, global matrices, load vector, B field and the linear solve
against the oracle's C restatement (oracle/femeko_oracle.c, or_nedelec_*)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

import femeko_gpu as fg
import oracle as O


def mesh_and_fields(n=3, seed=6):
    m = fg.box_tet_mesh(n, seed=seed, order=2, plate=((-3.0, 3.0), (-3.0, 3.0), (-3.0, 3.0)))
    assert np.any(m.elementID == 2)
    rng = np.random.default_rng(seed)
    nu = np.where(m.elementID == 2, 1.0 / 500.0, 1.0) * rng.uniform(0.9, 1.1, m.nt)
    return m, rng, nu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_edge_numbering_matches_reference_rule():
    m = fg.box_tet_mesh(2, seed=1, order=2)
    e1, n1 = fg.nedelec_edges(m)
    e2, n2 = O.nedelec_edges(m)
    assert n1 == n2 and np.array_equal(e1, e2)
    first = e1.T.ravel()
    seen = first[np.sort(np.unique(first, return_index=True)[1])]
    assert np.array_equal(seen, np.arange(n1))          # first appearance order


@pytest.mark.gpu
def test_nedelec_matrices_parity():
    m, rng, nu = mesh_and_fields()
    assert rel(fg.nedelecLocalStiffness(m), O.nedelecLocalStiffness(m)) < 1e-11
    Ag, Ao = fg.nedelecStiffness(m, nu), O.nedelecStiffness(m, nu)
    assert Ag.shape == Ao.shape and np.array_equal(Ag.indptr, Ao.indptr) and np.array_equal(Ag.indices, Ao.indices)
    assert rel(Ag.data, Ao.data) < 1e-11
    Bf = rng.normal(size=(3, m.nt))
    B = np.linalg.norm(Bf, axis=0)
    B[3] = 0.0
    dnu = -rng.uniform(0.1, 1.0, m.nt)
    Tg, To = fg.nedelecTangentialStiffness(m, dnu, Bf, B), O.nedelecTangentialStiffness(m, dnu, Bf, B)
    assert np.array_equal(Tg.indices, To.indices) and rel(Tg.data, To.data) < 1e-11
    Bext = np.array([0.5, 0.0, 0.0])
    assert rel(fg.nedelec_load(m, Bext), O.nedelec_load(m, Bext)) < 1e-11
    u = rng.normal(size=Ag.shape[0])
    (Bg, ng), (Bo, no) = fg.nedelec_bfield(m, u), O.nedelec_bfield(m, u)
    assert rel(Bg, Bo) < 1e-11 and rel(ng, no) < 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64"])
def test_nedelec_linear_solve(precision):
    """The curl-curl system is singular but consistent: u is one solution, B = curl u
    per element is unique; compare B with the oracle's CG solution."""
    m, _, nu = mesh_and_fields(n=4)
    Bext = np.array([0.5, 0.1, -0.2])
    u, Bf, B, st = fg.nedelec_linear(m, Bext, nu, precision=precision, rtol=1e-12)
    assert st["converged"]
    A, rhs = O.nedelecStiffness(m, nu), O.nedelec_load(m, Bext)
    assert np.linalg.norm(A @ u - rhs) <= 1e-10 * np.linalg.norm(rhs)
    uo, info = spla.cg(A, rhs, rtol=1e-13, maxiter=20000)
    # mixed precision: FP32 inner CG in FP64 refinement, finished in FP64 where the
    # FP32 iterations stall on this singular system; the same B
    u2, Bf2, _, st2 = fg.nedelec_linear(m, Bext, nu, precision="mixed", rtol=1e-12)
    assert st2["converged"] and np.linalg.norm(A @ u2 - rhs) <= 1e-10 * np.linalg.norm(rhs)
    assert rel(Bf2, Bf) < 1e-8
    Bo, _ = O.nedelec_bfield(m, uo)
    assert rel(Bf, Bo) < 1e-7
    assert np.allclose(B, np.linalg.norm(Bf, axis=0), rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_nedelec_handle_errors():
    m, _, _ = mesh_and_fields(n=2)
    g = fg.edge_mesh(m)
    with pytest.raises(RuntimeError):       # nodal element matrices refuse an edge handle
        fg.L.check(fg.L.lib().fg_stiffness(g.h, None, fg.L.ptr(np.zeros(g.nnz))))
    p1 = fg.box_tet_mesh(2, seed=1)
    with pytest.raises(RuntimeError):       # edge routines refuse a nodal handle
        fg.L.check(fg.L.lib().fg_nedelec_load(fg.gpu_mesh(p1).h, fg.L.ptr(np.ones(3)), fg.L.ptr(np.zeros(p1.nv))))


def iron_curve():
    """A smooth relative-reluctance curve nu(B) of a soft iron (0.002 at low field,
    saturating towards 1), 40 points on 0..3 T."""
    b = np.linspace(0.0, 3.0, 40)
    q = (b / 1.8) ** 6
    return b, 0.002 + 0.998 * q / (1.0 + q)


def test_nedelec_spline_matches_scipy_not_a_knot():
    b, nu = iron_curve()
    spl, spl_dnu = O.nedelec_splines(b, nu)
    assert np.allclose(spl(b), nu, rtol=0, atol=1e-15)
    assert spl(-1.0) == nu[0] and spl(9.0) == nu[-1]
    g = O.fd_gradient(b, nu)
    assert np.allclose(spl_dnu(b), g, rtol=0, atol=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nedelec_newton_parity(precision):
    m, _, _ = mesh_and_fields(n=4)
    b, nu_tab = iron_curve()
    nl = (m.elementID == 2).astype(np.uint8)
    Bext = np.array([0.8, 0.0, 0.0])
    u, Bf, B, nu, it, st = fg.nedelec_newton(m, Bext, b, nu_tab, nonlinear=nl, tol=1e-6, precision=precision,
                                             rtol=1e-11)
    uo, Bfo, Bo, nuo, ito = O.nedelec_newton(m, Bext, b, nu_tab, nl, tol=1e-6, cg_rtol=1e-11)
    assert st["converged"] and abs(it - ito) <= 1 and it >= 3, (st, it, ito)
    assert rel(Bf, Bfo) < 1e-5 and rel(nu, nuo) < 1e-5
    spl, _ = O.nedelec_splines(b, nu_tab)
    assert rel(nu[nl == 1], spl(B[nl == 1])) < 1e-12        # the device spline is scipy's not-a-knot cubic
    assert np.all(nu[nl == 0] == 1.0)
