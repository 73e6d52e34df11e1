"""The reference's own ccall entry point scalarPotential
(Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:49-95) against the oracle's
restatement of magnetostatics() (:5-38): the linear Neumann problem with the
boundary flux of a uniform field, solved from u = 0 with Jacobi-PCG.

The potential is unique up to a constant (the system is singular and consistent), so
u is compared after removing the diagonal-weighted mean that a PCG from zero keeps at
zero; H = -grad u is compared directly.
"""
import dataclasses

import numpy as np
import pytest

import femeko_gpu as fg
import femeko_gpu._lib as L
import oracle as O

pytestmark = pytest.mark.gpu

MU0 = fg.MU0


def _centre(u, K):
    d = K.diagonal()
    return u - (d * u).sum() / d.sum()


def _plate(n=10, seed=4):
    m = fg.box_tet_mesh(n, seed=seed)
    mu = np.where(m.elementID == 2, 3.0 * MU0, MU0)   # run.jl:58-59: mu0 (1 + 2) inside
    return m, mu


@pytest.mark.parametrize("reference_call", [True, False])
def test_scalar_potential_matches_oracle(reference_call):
    m, mu = _plate()
    Hext = np.array([1.0, 0.0, 0.0])                   # run.jl:19
    ug, st = fg.scalarPotential(m, mu, Hext, 1, reference_call=reference_call)
    uo, it, rr = O.scalarPotential(m, mu, Hext, 1, tol=1e-14)
    K = O.stiffnessMatrix(m, mu)
    if reference_call:
        assert st["status"] == L.FG_OK and L.lib().fg_last_error() == b""
    else:
        assert st["converged"]
    a, b = _centre(ug, K), _centre(uo, K)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-8
    Hg, Ho = O.hfield(m, ug), O.hfield(m, uo)
    assert np.linalg.norm(Hg - Ho) / np.linalg.norm(Ho) < 1e-8
    # the residual of the reference's system itself
    RHS = O.BoundaryIntegral(m, Hext, (1,))
    assert np.linalg.norm(K @ ug + RHS) / np.linalg.norm(RHS) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_scalar_potential_uniform_mu_is_linear(precision):
    """Patch test: with a uniform mu the potential is -Hext.x / mu + c exactly."""
    m = fg.box_tet_mesh(6, seed=9)
    Hext = np.array([0.3, -1.1, 0.5])
    ug, st = fg.scalarPotential(m, np.full(m.nt, 2.0), Hext, 1, precision=precision)
    exact = -(Hext[:, None] * m.p).sum(axis=0) / 2.0
    d = ug - exact
    assert st["converged"]
    assert np.abs(d - d.mean()).max() < 1e-9 * np.abs(exact).max()


def test_scalar_potential_other_shell_id_and_caller_volumes():
    """Faces with another boundary id carry no flux; the stiffness uses the caller's
    VE (src/FEMc.cpp:74-96), here scaled by 2 on every element: u halves."""
    m, mu = _plate(8, 2)
    Hext = np.array([0.0, 1.0, 0.0])
    u1, _ = fg.scalarPotential(m, mu, Hext, 1, reference_call=True)
    u0, _ = fg.scalarPotential(m, mu, Hext, 7, reference_call=True)    # no face has id 7: RHS = 0
    assert np.abs(u0).max() == 0.0
    m2 = dataclasses.replace(m, VE=2.0 * m.VE)
    u2, _ = fg.scalarPotential(m2, mu, Hext, 1, reference_call=True)
    K = O.stiffnessMatrix(m, mu)
    a, b = _centre(u2, K), _centre(u1, K)
    assert np.linalg.norm(a - 0.5 * b) / np.linalg.norm(0.5 * b) < 1e-8


def test_scalar_potential_error_leaves_u_and_reports():
    """A node index outside the mesh: nothing is thrown through the void function; the
    status and message are kept and u is left as it was."""
    import ctypes as C
    m, mu = _plate(4, 1)
    lib = L.lib()
    t = np.ascontiguousarray(m.t.T, dtype=np.int32)
    t[3, 2] = m.nv + 10
    sT = np.ascontiguousarray(m.surfaceT.T, dtype=np.int32)
    u = np.full(m.nv, 7.0)
    args = [L.ptr(u), L.ptr(np.ascontiguousarray(m.p.T)), L.ptr(t), L.ptr(sT),
            L.ptr(np.ascontiguousarray(m.normal.T)), C.c_int(m.nv), C.c_int(m.nt), C.c_int(m.ns),
            L.ptr(np.ascontiguousarray(m.VE)), L.ptr(np.ascontiguousarray(mu)), L.ptr(np.array([1.0, 0, 0])),
            C.c_int(0)]
    lib.scalarPotential(*args)
    assert lib.fg_scalar_potential_status() == L.FG_BAD_MESH
    assert lib.fg_last_error() != b""
    assert np.all(u == 7.0)
    # the next good call clears both
    fg.scalarPotential(m, mu, np.array([1.0, 0, 0]), 1, reference_call=True)
    assert lib.fg_scalar_potential_status() == L.FG_OK and lib.fg_last_error() == b""
