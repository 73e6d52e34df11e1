"""GPU backward-Euler heat (fg_heat_be) against the FP64 oracle, compared every 10th
step, in FP64 and in mixed precision (FP32 operator/CG inside FP64 refinement)."""
import numpy as np
import pytest

import femeko_gpu as fg
import oracle as O

pytestmark = pytest.mark.gpu


def heat_case(n=8, seed=6):
    m = fg.box_tet_mesh(n, seed=seed)
    rng = np.random.default_rng(3)
    kappa = np.exp(rng.normal(size=m.nt))          # lognormal(0, 1)
    x0 = np.array([0.7, -0.4, 0.3])                  # bump centre (interior)
    T0 = np.exp(-(((m.p - x0[:, None]) ** 2).sum(axis=0)) / 0.5 ** 2)
    return m, kappa, T0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_heat_be_every_10th_step(precision):
    m, kappa, T0 = heat_case()
    T, snaps, st = fg.heat_be(m, T0, kappa, rho_c=1.0, dt=1e-3, nsteps=30, every=10, precision=precision,
                              rtol=1e-10)
    To, so, _ = O.heat_be(m, T0, kappa, 1.0, 1e-3, 30, cg_tol=1e-12, every=10)
    assert st["converged"]
    assert snaps.shape == so.shape == (3, m.nv)
    for k in range(3):
        assert np.linalg.norm(snaps[k] - so[k]) / np.linalg.norm(so[k]) < 1e-8, k
    assert np.array_equal(T, snaps[-1])
    assert np.all(T[m.dirichlet_mask().astype(bool)] == 0.0)


def test_heat_be_rho_c_and_zero_steps():
    m, kappa, T0 = heat_case(n=6)
    T, snaps, st = fg.heat_be(m, T0, kappa, rho_c=2.5, dt=2e-3, nsteps=5, every=5, precision="fp64", rtol=1e-12)
    To, so, _ = O.heat_be(m, T0, kappa, 2.5, 2e-3, 5, cg_tol=1e-13, every=5)
    assert np.linalg.norm(T - To) / np.linalg.norm(To) < 1e-9
    T1, _, _ = fg.heat_be(m, T0, kappa, nsteps=0, every=0)
    fx = m.dirichlet_mask().astype(bool)
    assert np.array_equal(T1[~fx], T0[~fx]) and np.all(T1[fx] == 0.0)
