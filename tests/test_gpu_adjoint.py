"""GPU adjoint dJ/dmur (fg_adjoint_dJdmu) against the FP64 CPU adjoint of the oracle
and against central finite differences of J.

J = volume-weighted mean of H_x over the elements with centroid inside a ball.
"""
import numpy as np
import pytest

import femeko_gpu as fg
import oracle as O

pytestmark = pytest.mark.gpu

MU0 = fg.MU0


def linear_case(n=8, seed=9, radius=2.0):
    m = fg.box_tet_mesh(n, seed=seed)
    rng = np.random.default_rng(5)
    mur = rng.uniform(1, 1000, m.nt)
    c = m.centroids()
    target = (np.sqrt((c * c).sum(axis=0)) < radius).astype(np.uint8)
    u0 = -m.p[0].copy()
    return m, mur, target, u0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_linear_matches_cpu_adjoint(precision):
    m, mur, target, u0 = linear_case()
    J, grad, u, st = fg.adjoint_dJdmu(m, mur, u0, target, precision=precision, rtol=1e-12)
    assert st["converged"]
    uo, _, _ = O.linear_magnetostatics(m, u0, mur * MU0, cg_tol=1e-14)
    Jo = O.objective_hx(m, target, uo)
    go, _ = O.adjoint(m, target, mur * MU0, uo, cg_tol=1e-14)
    go = go * MU0   # per relative permeability
    assert abs(J - Jo) <= 1e-10 * abs(Jo)
    assert np.linalg.norm(u - uo) / np.linalg.norm(uo) < 1e-10
    assert np.abs(grad - go).max() <= 1e-8 * np.abs(go).max()


def test_adjoint_linear_central_differences():
    """Central differences with relative step 1e-6 on 32 random elements (FP64 CPU
    solves of the perturbed problems to 1e-14), drawn among the elements whose
    sensitivity is at least 1% of the largest (below that the difference quotient
    sinks into rounding).  J is linear in u, so J(u+) - J(u-) is evaluated as
    J(u+ - u-), which avoids cancelling two O(1) values."""
    m, mur, target, u0 = linear_case()
    J, grad, u, st = fg.adjoint_dJdmu(m, mur, u0, target, precision="mixed", rtol=1e-12)
    rng = np.random.default_rng(11)
    scale = np.abs(grad).max()
    pool = np.flatnonzero(np.abs(grad) >= 1e-2 * scale)
    assert pool.size >= 32
    for k in rng.choice(pool, 32, replace=False):
        d = 1e-6 * mur[k]
        us = []
        for s in (+1, -1):
            mu2 = mur * MU0
            mu2[k] = (mur[k] + s * d) * MU0
            u2, _, _ = O.linear_magnetostatics(m, u0, mu2, cg_tol=1e-14)
            us.append(u2)
        fd = O.objective_hx(m, target, us[0] - us[1]) / (2 * d)
        assert abs(fd - grad[k]) <= 1e-5 * abs(grad[k]), (k, fd, grad[k])


def test_adjoint_nonlinear_newton_tangent():
    """Through the converged Newton Jacobian (Froehlich plate, mur elsewhere)."""
    m = fg.box_tet_mesh(10, seed=2)
    nl = (m.elementID == 2).astype(np.uint8)
    rng = np.random.default_rng(3)
    mur = np.where(nl == 1, 1.0, rng.uniform(1, 1000, m.nt))
    u0 = -(np.array([8e4, 0.0, 0.0])[:, None] * m.p).sum(axis=0)
    c = m.centroids()
    target = (np.sqrt((c * c).sum(axis=0)) < 1.5).astype(np.uint8)
    J, grad, u, st = fg.adjoint_dJdmu(m, mur, u0, target, nl=nl, precision="fp64", rtol=1e-12, tol_update=1e-12,
                                      forcing="fixed", inner_rtol=1e-12)
    assert st["converged"] and st["newton_iters"] > 1
    uo, Ho, muo, so = O.newton(m, u0, nl, mur * MU0, 1.2e6, 500.0, tol_update=1e-12, cg_tol=1e-13)
    assert so["converged"]
    h = np.sqrt((Ho * Ho).sum(axis=0))
    dmu = np.array([O.froehlich(hk, 1.2e6, 500.0)[1] if f else 0.0 for hk, f in zip(h, nl)])
    go, _ = O.adjoint(m, target, muo, uo, H=Ho, dmu=dmu, cg_tol=1e-14)
    go = go * MU0
    assert abs(J - O.objective_hx(m, target, uo)) <= 1e-9 * abs(J)
    assert np.abs(grad - go).max() <= 1e-7 * np.abs(go).max()
    # linear elements carry the sensitivity; Froehlich elements have mur = 1 here
    assert np.abs(grad[nl == 0]).max() > 0
