"""Many independent linear magnetostatic problems in one persistent launch
(fg_batch_magnetostatics_linear) against the oracle's per-mesh solve."""
import numpy as np
import pytest

import femeko_gpu as fg
import oracle as O

pytestmark = pytest.mark.gpu


def batch_case(count, lo, hi, seed=7):
    rng = np.random.default_rng(seed)
    meshes, mus, u0s = [], [], []
    for k in range(count):
        n = int(rng.integers(lo, hi + 1))
        m = fg.box_tet_mesh(n, seed=100 + k)
        meshes.append(m)
        mus.append(rng.uniform(1, 1000, m.nt) * fg.MU0)
        u0s.append(-m.p[0].copy())
    return meshes, mus, u0s


def test_batch_matches_single_solves():
    meshes, mus, u0s = batch_case(12, 3, 9)
    us, its, st = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10)
    assert st["problems"] == 12 and st["converged"] == 12
    assert st["max_iterations"] == its.max() and st["total_iterations"] == its.sum()
    for m, mu, u0, u, it in zip(meshes, mus, u0s, us, its):
        uo, Ho, _ = O.linear_magnetostatics(m, u0, mu, cg_tol=1e-13)
        assert it > 0
        assert np.linalg.norm(u - uo) / np.linalg.norm(uo) < 1e-8
        fx = m.dirichlet_mask().astype(bool)
        assert np.array_equal(u[fx], u0[fx])


def test_batch_sixty_four_uneven_meshes_twice():
    """64 problems of uneven size; a second call on the same handles gives the same
    answer (the launch and its graph are rebuilt per call)."""
    meshes, mus, u0s = batch_case(64, 4, 12, seed=3)
    us1, its1, st1 = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-9)
    us2, its2, st2 = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-9)
    assert st1["converged"] == 64 and np.array_equal(its1, its2)
    for a, b in zip(us1, us2):
        assert np.array_equal(a, b)
    k = int(np.argmax([m.nv for m in meshes]))
    uo, _, _ = O.linear_magnetostatics(meshes[k], u0s[k], mus[k], cg_tol=1e-12)
    assert np.linalg.norm(us1[k] - uo) / np.linalg.norm(uo) < 1e-7


def test_batch_mixed_precision_matches_single_solves():
    """FP32 PCG inside FP64 refinement on each cluster reaches the FP64 answer."""
    meshes, mus, u0s = batch_case(12, 3, 14, seed=11)
    us, its, st = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10, precision="mixed")
    assert st["problems"] == 12 and st["converged"] == 12
    assert st["max_refinements"] >= 2          # inner solves stop at 1e-5: two or more refinements
    assert st["max_iterations"] == its.max() and st["total_iterations"] == its.sum()
    u64, its64, st64 = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10)
    assert st64["max_refinements"] == 0
    for m, mu, u0, u, v in zip(meshes, mus, u0s, us, u64):
        uo, _, _ = O.linear_magnetostatics(m, u0, mu, cg_tol=1e-13)
        assert np.linalg.norm(u - uo) / np.linalg.norm(uo) < 1e-8
        assert np.linalg.norm(v - uo) / np.linalg.norm(uo) < 1e-8
        fx = m.dirichlet_mask().astype(bool)
        assert np.array_equal(u[fx], u0[fx])
    us2, its2, _ = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10, precision="mixed")
    assert np.array_equal(its, its2)
    for a, b in zip(us, us2):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_iteration_cap_is_reported(precision):
    meshes, mus, u0s = batch_case(4, 6, 9, seed=5)
    us, its, st = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-12, maxiter=7, precision=precision)
    assert st["converged"] == 0
    assert (its <= 7).all() and its.max() == 7
    for u in us:
        assert np.isfinite(u).all()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_triangles_and_tetrahedra_together(precision):
    """P1 triangle and tetrahedron meshes in one launch, each against a direct solve
    of the oracle's stiffness matrix on the free rows."""
    import scipy.sparse.linalg as spla
    rng = np.random.default_rng(21)
    meshes = [fg.box_tri_mesh(24, seed=1), fg.box_tet_mesh(7, seed=2), fg.box_tri_mesh(10, seed=3)]
    mus = [rng.uniform(1, 1000, m.nt) * fg.MU0 for m in meshes]
    u0s = [-m.p[0].copy() for m in meshes]
    us, its, st = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-11, precision=precision)
    assert st["problems"] == 3 and st["converged"] == 3
    for m, mu, u0, u in zip(meshes, mus, u0s, us):
        K = (O.stiffnessMatrix2D(m, mu) if m.t.shape[0] == 3 else O.stiffnessMatrix(m, mu)).tocsr()
        fx = m.dirichlet_mask().astype(bool)
        fr = ~fx
        ref = u0.copy()
        ref[fr] = spla.spsolve(K[fr][:, fr].tocsc(), -(K[fr][:, fx] @ u0[fx]))
        assert np.linalg.norm(u - ref) / np.linalg.norm(ref) < 1e-8
        assert np.array_equal(u[fx], u0[fx])


def test_batch_single_problem_mixed_matches_fp64():
    """One problem alone (the largest cluster) in both precisions."""
    meshes, mus, u0s = batch_case(1, 16, 16, seed=13)
    um, itm, stm = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10, precision="mixed")
    ud, itd, std = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10)
    assert stm["converged"] == 1 and std["converged"] == 1
    assert stm["cluster_ctas"] == std["cluster_ctas"] and stm["cluster_ctas"] in (8, 16)
    assert np.linalg.norm(um[0] - ud[0]) / np.linalg.norm(ud[0]) < 1e-8
