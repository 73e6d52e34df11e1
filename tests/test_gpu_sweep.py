"""Field sweep as one multi-right-hand-side CG (fg_magnetostatics_sweep) against one
oracle solve per applied field."""
import numpy as np
import pytest

import femeko_gpu as fg
import oracle as O

pytestmark = pytest.mark.gpu


def sweep_fields(nf, seed=4):
    rng = np.random.default_rng(seed)
    h = rng.uniform(-1e5, 1e5, nf)
    th = rng.uniform(0, np.pi, nf)
    return np.stack([h * np.cos(th), h * np.sin(th), np.zeros(nf)], axis=1)


@pytest.mark.parametrize("nf", [5, 40, 256])
def test_sweep_matches_per_field_solves(nf):
    m = fg.box_tet_mesh(7, seed=12)
    mu = np.where(m.elementID == 2, 1000.0, 1.0) * fg.MU0
    H0 = sweep_fields(nf)
    U, st = fg.magnetostatics_sweep(m, mu, H0, rtol=1e-10)
    assert st["converged"] and U.shape == (m.nv, nf)
    check = range(nf) if nf <= 40 else np.random.default_rng(1).choice(nf, 12, replace=False)
    fx = m.dirichlet_mask().astype(bool)
    for c in check:
        u0 = -(H0[c][:, None] * m.p).sum(axis=0)
        uo, _, _ = O.linear_magnetostatics(m, u0, mu, cg_tol=1e-13)
        assert np.linalg.norm(U[:, c] - uo) / np.linalg.norm(uo) < 1e-8, c
        assert np.allclose(U[fx, c], u0[fx], rtol=0, atol=1e-9 * np.abs(u0).max())


def test_sweep_is_linear_in_the_field():
    """Potentials of a combination of fields equal the combination of potentials."""
    m = fg.box_tet_mesh(6, seed=2)
    mu = np.random.default_rng(0).uniform(1, 1000, m.nt) * fg.MU0
    H0 = np.array([[1e4, 0, 0], [0, 1e4, 0], [3e4, -2e4, 0]])
    U, st = fg.magnetostatics_sweep(m, mu, H0, rtol=1e-12)
    comb = 3 * U[:, 0] - 2 * U[:, 1]
    assert np.linalg.norm(U[:, 2] - comb) / np.linalg.norm(comb) < 1e-9
