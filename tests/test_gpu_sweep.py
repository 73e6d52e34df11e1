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


@pytest.mark.parametrize("method", ["block", "per_field"])
@pytest.mark.parametrize("nf", [5, 40, 256])
def test_sweep_matches_per_field_solves(nf, method):
    m = fg.box_tet_mesh(7, seed=12)
    mu = np.where(m.elementID == 2, 1000.0, 1.0) * fg.MU0
    H0 = sweep_fields(nf)
    U, st = fg.magnetostatics_sweep(m, mu, H0, rtol=1e-10, method=method)
    assert st["converged"] and U.shape == (m.nv, nf)
    if method == "block":
        assert st["rank"] == 2          # h (cos t, sin t, 0): the x-y plane
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


@pytest.mark.parametrize("kind,rank", [("one_direction", 1), ("three_d", 3), ("with_zero_fields", 2)])
def test_block_sweep_rank_reduction(kind, rank):
    """The block method solves one problem per independent field direction (the rank
    of H0) and combines them; each field still matches its own oracle solve."""
    m = fg.box_tet_mesh(6, seed=4)
    mu = np.random.default_rng(8).uniform(1, 1000, m.nt) * fg.MU0
    rng = np.random.default_rng(9)
    if kind == "one_direction":
        H0 = np.outer(rng.uniform(-1e5, 1e5, 20), [0.6, -0.8, 0.0])
    elif kind == "three_d":
        H0 = rng.normal(size=(20, 3)) * 1e4
    else:
        H0 = sweep_fields(20)
        H0[[3, 7]] = 0.0
    U, st = fg.magnetostatics_sweep(m, mu, H0, rtol=1e-10)
    assert st["converged"] and st["rank"] == rank
    for c in range(0, 20, 3):
        u0 = -(H0[c][:, None] * m.p).sum(axis=0)
        uo, _, _ = O.linear_magnetostatics(m, u0, mu, cg_tol=1e-13)
        if np.abs(uo).max() == 0.0:
            assert np.abs(U[:, c]).max() == 0.0
        else:
            assert np.linalg.norm(U[:, c] - uo) / np.linalg.norm(uo) < 1e-8, c


def test_block_and_per_field_agree():
    m = fg.box_tet_mesh(8, seed=3)
    mu = np.random.default_rng(12).uniform(1, 1000, m.nt) * fg.MU0
    H0 = sweep_fields(64, seed=6)
    Ub, sb = fg.magnetostatics_sweep(m, mu, H0, rtol=1e-11, method="block")
    Up, sp_ = fg.magnetostatics_sweep(m, mu, H0, rtol=1e-11, method="per_field")
    assert sb["converged"] and sp_["converged"]
    assert np.abs(Ub - Up).max() <= 1e-9 * np.abs(Up).max()
