"""The benchmark configurations at their stated sizes (or, where a full-size oracle
run takes minutes, the largest size the oracle finishes in well under two minutes
on 16 host cores, named in the test), GPU against the FP64 oracle.

C1  linear plate, 24^3 cells, mu_r = 1000, Jacobi-PCG to 1e-10
C2  backward-Euler heat, 64^3 cells, 100 steps, every 10th step, FP64 and mixed
C3  Froehlich-plate Newton, 48^3 cells here (96^3 is compared on every benchmark
    run, accuracy_vs_oracle), both precisions, H, u, mu and the energy
C4a 256 applied fields on the 48^3-cell plate, a sample of fields per oracle solve
C4b 64 meshes of 8..40 cells per side in one launch, a sample per oracle solve
C5  adjoint dJ/dmu_r on 64^3 cells against the FP64 CPU adjoint and central
    differences on 32 elements; the Newton-tangent adjoint on the 64^3 Froehlich plate
"""
import numpy as np
import pytest

import femeko_gpu as fg
import oracle as O

pytestmark = pytest.mark.gpu

MU0 = fg.MU0
SEED = 20261203
MS, HK = 1.2e6, 500.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module", autouse=True)
def all_host_threads():
    import os
    O.set_threads(os.cpu_count() or 1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c1_linear_plate_24cube(precision):
    m = fg.box_tet_mesh(24, seed=SEED)
    mu = np.where(m.elementID == 2, 1000.0, 1.0) * MU0
    u0 = -m.p[0].copy()                                   # H0 = (1, 0, 0)
    ug, Hg, st = fg.magnetostatics_linear(m, mu, u0, precision=precision, rtol=1e-10)
    uo, Ho, it = O.linear_magnetostatics(m, u0, mu, cg_tol=1e-13)
    assert st["converged"] and st["relres"] <= 1e-10
    assert rel(Hg, Ho) < 1e-8 and rel(ug, uo) < 1e-8


@pytest.fixture(scope="module")
def heat64():
    m = fg.box_tet_mesh(64, seed=SEED)
    rng = np.random.default_rng(SEED)
    kappa = np.exp(rng.normal(size=m.nt))               # lognormal(0, 1)
    x0 = rng.uniform(-2.5, 2.5, 3)                      # bump centre, seeded interior point
    T0 = np.exp(-(((m.p - x0[:, None]) ** 2).sum(axis=0)) / 0.5 ** 2)
    To, so, _ = O.heat_be(m, T0, kappa, 1.0, 1e-3, 100, cg_tol=1e-13, every=10)
    return m, kappa, T0, so


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c2_heat_64cube_100_steps_every_10th(heat64, precision):
    m, kappa, T0, so = heat64
    T, snaps, st = fg.heat_be(m, T0, kappa, rho_c=1.0, dt=1e-3, nsteps=100, every=10, precision=precision,
                              rtol=1e-10)
    assert st["converged"] and snaps.shape == (10, m.nv)
    errs = [rel(snaps[k], so[k]) for k in range(10)]
    assert max(errs) < 1e-8, errs


@pytest.fixture(scope="module")
def newton48():
    m = fg.box_tet_mesh(48, seed=SEED)
    nl = (m.elementID == 2).astype(np.uint8)
    mu_lin = np.full(m.nt, MU0)
    u0 = -(np.array([8e4, 0.0, 0.0])[:, None] * m.p).sum(axis=0)
    uo, Ho, muo, so = O.newton(m, u0, nl, mu_lin, MS, HK, tol_update=1e-8, line_search="residual", forcing="ew",
                               eta_min=1e-2, eta_max=0.3, picard_steps=2)
    assert so["converged"]
    return m, nl, mu_lin, u0, uo, Ho, muo, O.energy(m, Ho, nl, mu_lin, MS, HK)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c3_froehlich_newton_48cube(newton48, precision):
    m, nl, mu_lin, u0, uo, Ho, muo, Wo = newton48
    ug, Hg, mug, st = fg.newton_magnetostatics(m, nl, mu_lin, u0, precision=precision)
    assert st["converged"]
    assert rel(Hg, Ho) < 1e-8 and rel(ug, uo) < 1e-8
    assert np.abs(mug - muo).max() / muo.max() < 1e-8
    assert abs(st["energy"] - Wo) / Wo < 1e-8


def test_c4a_sweep_48cube_256_fields():
    m = fg.box_tet_mesh(48, seed=SEED)
    mu = np.where(m.elementID == 2, 1000.0, 1.0) * MU0
    rng = np.random.default_rng(SEED)
    h, th = rng.uniform(-1e5, 1e5, 256), rng.uniform(0, np.pi, 256)
    H0 = np.stack([h * np.cos(th), h * np.sin(th), np.zeros(256)], axis=1)
    U, st = fg.magnetostatics_sweep(m, mu, H0, rtol=1e-10)
    assert st["converged"] and U.shape == (m.nv, 256)
    for c in np.random.default_rng(2).choice(256, 6, replace=False):
        u0 = -(H0[c][:, None] * m.p).sum(axis=0)
        uo, _, _ = O.linear_magnetostatics(m, u0, mu, cg_tol=1e-13)
        assert rel(U[:, c], uo) < 1e-8, c


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c4b_batch_64_meshes_8_to_40_cells(precision):
    rng = np.random.default_rng(SEED)
    ns = rng.integers(8, 41, 64)
    meshes = [fg.box_tet_mesh(int(n), seed=SEED + k) for k, n in enumerate(ns)]
    mus = [rng.uniform(1, 1000, m.nt) * MU0 for m in meshes]
    u0s = [-m.p[0].copy() for m in meshes]
    us, its, st = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10, precision=precision)
    assert st["problems"] == 64 and st["converged"] == 64
    order = np.argsort(ns)
    sample = sorted({int(order[0]), int(order[-1]), int(order[32]), *map(int, np.random.default_rng(5).choice(64, 3,
                                                                                                             False))})
    for k in sample:
        uo, _, _ = O.linear_magnetostatics(meshes[k], u0s[k], mus[k], cg_tol=1e-13)
        assert rel(us[k], uo) < 1e-8, (k, int(ns[k]))


@pytest.fixture(scope="module")
def adjoint64():
    m = fg.box_tet_mesh(64, seed=SEED)
    rng = np.random.default_rng(SEED)
    mur = rng.uniform(1, 1000, m.nt)
    c = m.centroids()
    target = (np.sqrt((c * c).sum(axis=0)) < 0.5).astype(np.uint8)
    u0 = -m.p[0].copy()
    return m, mur, target, u0


def test_c5_adjoint_64cube_linear_vs_cpu_adjoint_and_central_differences(adjoint64):
    m, mur, target, u0 = adjoint64
    J, grad, u, st = fg.adjoint_dJdmu(m, mur, u0, target, precision="mixed", rtol=1e-12)
    assert st["converged"]
    # the oracle's FP64 PCG to 1e-12 (tighter stalls at this size: mu_r spans 1..1000)
    uo, _, _ = O.linear_magnetostatics(m, u0, mur * MU0, cg_tol=1e-12, cg_maxit=50000)
    go, _ = O.adjoint(m, target, mur * MU0, uo, cg_tol=1e-12, cg_maxit=50000)
    go = go * MU0
    assert abs(J - O.objective_hx(m, target, uo)) <= 1e-9 * abs(J)
    assert np.abs(grad - go).max() <= 1e-7 * np.abs(go).max()
    # central differences with relative step 1e-6 on 32 elements whose sensitivity is
    # at least 1% of the largest
    fd = central_differences_linear(m, mur, u, target, grad, rel_step=1e-6, count=32, seed=11)
    for k, val in fd:
        assert abs(val - grad[k]) <= 1e-5 * abs(grad[k]), (k, val, grad[k])


def _element_stiffness(m, k):
    """VE grad(phi_a).grad(phi_b) of element k (unit coefficient), from its vertices."""
    P = np.vstack([np.ones(4), m.p[:, m.t[:4, k]]])
    G = np.linalg.inv(P)[:, 1:4]
    return m.VE[k] * (G @ G.T)


def central_differences_linear(m, mur, u, target, grad, rel_step, count, seed):
    """dJ/dmur_k by central differences of the linear Dirichlet problem.  The
    perturbed solutions are u + du with A(mu +- d) du = -(+-d) dA/dmur_k u on the free
    nodes: the right-hand side is local to element k and exact, where forming
    b - A(mu +- d) u from the whole field would lose about eps |b| to cancellation (as
    much as the perturbation itself at small steps).  J is linear in u."""
    import scipy.sparse as sp
    fixed = m.dirichlet_mask().astype(bool)
    free = np.flatnonzero(~fixed)
    Kff = fg.stiffnessMatrix(m, mur * MU0).tocsr()[free][:, free].tocsc()
    pos = np.full(m.nv, -1)
    pos[free] = np.arange(free.size)
    rng = np.random.default_rng(seed)
    pool = np.flatnonzero(np.abs(grad) >= 1e-2 * np.abs(grad).max())
    assert pool.size >= count
    out = []
    for k in rng.choice(pool, count, replace=False):
        nodes = m.t[:4, k]
        Ek = MU0 * _element_stiffness(m, k)
        g = Ek @ u[nodes]
        keep = pos[nodes] >= 0
        fi = pos[nodes][keep]
        P = sp.csc_matrix((Ek[np.ix_(keep, keep)].ravel(), (np.repeat(fi, fi.size), np.tile(fi, fi.size))),
                          shape=Kff.shape)
        d = rel_step * mur[k]
        dus = []
        for s in (+1.0, -1.0):
            rhs = np.zeros(free.size)
            rhs[fi] = -s * d * g[keep]
            x = fg.cg(Kff + s * d * P, rhs, reltol=1e-12, precision="fp64")
            du = np.zeros(m.nv)
            du[free] = x
            dus.append(du)
        out.append((int(k), O.objective_hx(m, target, dus[0] - dus[1]) / (2 * d)))
    return out


def test_c5_adjoint_64cube_through_newton_tangent():
    m = fg.box_tet_mesh(64, seed=SEED)
    nl = (m.elementID == 2).astype(np.uint8)
    rng = np.random.default_rng(SEED)
    mur = np.where(nl == 1, 1.0, rng.uniform(1, 1000, m.nt))
    u0 = -(np.array([8e4, 0.0, 0.0])[:, None] * m.p).sum(axis=0)
    c = m.centroids()
    target = (np.sqrt((c * c).sum(axis=0)) < 0.5).astype(np.uint8)
    J, grad, u, st = fg.adjoint_dJdmu(m, mur, u0, target, nl=nl, precision="mixed", rtol=1e-12, tol_update=1e-12,
                                      forcing="fixed", inner_rtol=1e-12)
    assert st["converged"] and st["newton_iters"] > 1
    uo, Ho, muo, so = O.newton(m, u0, nl, mur * MU0, MS, HK, tol_update=1e-11, line_search="residual", forcing="ew",
                               eta_min=1e-8, eta_max=0.1, picard_steps=2)
    assert so["converged"]
    h = np.sqrt((Ho * Ho).sum(axis=0))
    dmu = np.zeros(m.nt)
    for k in np.flatnonzero(nl):
        dmu[k] = O.froehlich(h[k], MS, HK)[1]
    go, _ = O.adjoint(m, target, muo, uo, H=Ho, dmu=dmu, cg_tol=1e-12, cg_maxit=50000)
    go = go * MU0
    assert abs(J - O.objective_hx(m, target, uo)) <= 1e-9 * abs(J)
    assert np.abs(grad - go).max() <= 1e-7 * np.abs(go).max()
