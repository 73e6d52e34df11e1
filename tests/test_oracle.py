"""Pins the CPU oracle: golden fixtures derived in exact arithmetic from the reference
formulas (tests/golden/make_golden.py) and the known answers of the maths.  CPU only."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle as O
from femeko_gpu.mesh import MESH, MU0, box_tet_mesh, box_tri_mesh, element_volumes, triangle_areas

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def gold():
    return json.load(open(os.path.join(GOLD, "element_matrices.json")))


def one_element_mesh(p, t, dim):
    p = np.asarray(p, dtype=np.float64).T
    if p.shape[0] == 2:
        p = np.vstack([p, np.zeros(p.shape[1])])
    t = np.asarray(t, dtype=np.int32).reshape(-1, 1)
    nvert = dim + 1
    VE = element_volumes(p, t[:4]) if dim == 3 else triangle_areas(p, t[:3])
    return MESH(order=1 if t.shape[0] == nvert else 2, dim=dim, p=p, t=t,
                surfaceT=np.zeros((4, 0), np.int32), elementID=np.ones(1, np.int32),
                InsideElements=np.zeros(0, np.int32), InsideNodes=np.zeros(0, np.int32), VE=VE,
                AE=np.zeros(0), normal=np.zeros((3, 0)), boundary_nodes=np.zeros(0, np.int32))


def dense(A):
    return np.asarray(sp.csc_matrix(A).todense())


def test_p1_tet_element(gold):
    g = gold["tet4_unit"]
    m = one_element_mesh(g["p"], [0, 1, 2, 3], 3)
    assert np.allclose(dense(O.stiffnessMatrix(m)), g["K"], rtol=0, atol=1e-15)
    assert np.allclose(dense(O.massMatrix(m)), g["M"], rtol=0, atol=1e-16)
    assert abs(O.element_volumes(m)[0] - g["VE"]) < 1e-16


def test_p1_tri_element(gold):
    g = gold["tri3_unit"]
    m = one_element_mesh(g["p"], [0, 1, 2], 2)
    assert np.allclose(dense(O.stiffnessMatrix2D(m)), g["K"], rtol=0, atol=1e-15)
    assert np.allclose(dense(O.massMatrix2D(m)), g["M"], rtol=0, atol=1e-16)


def test_p2_tet_element(gold):
    g = gold["tet10_unit"]
    m = one_element_mesh(g["p"], list(range(10)), 3)
    for shift in (False, True):
        assert np.allclose(dense(O.quadraticStiffnessMatrix(m, shift=shift)), g["K"], rtol=0, atol=1e-13)
    assert np.allclose(dense(O.quadraticMassMatrix(m, full_phi=True)), g["M_full"], rtol=0, atol=1e-15)
    assert np.allclose(dense(O.quadraticMassMatrix(m, full_phi=False)), g["M_linear_part"], rtol=0, atol=1e-15)


def test_p2_tri_element(gold):
    g = gold["tri6_unit"]
    m = one_element_mesh(g["p"], list(range(6)), 2)
    assert np.allclose(dense(O.quadraticStiffnessMatrix2D(m)), g["K"], rtol=0, atol=1e-13)
    assert np.allclose(dense(O.quadraticMassMatrix2D(m)), g["M"], rtol=0, atol=1e-14)


def test_kuhn2_global_stiffness():
    ref = json.load(open(os.path.join(GOLD, "kuhn2_stiffness.json")))
    m = box_tet_mesh(2, jitter=0.0)
    K = O.stiffnessMatrix(m)
    assert np.array_equal(K.indptr, ref["colptr"]) and np.array_equal(K.indices, ref["rowval"])
    assert np.abs(K.data - np.array(ref["data"])).max() < 1e-14
    # the chained sparse `+` drops exact zeros (src/FEM3D.jl:51)
    Kd = O.stiffnessMatrix(m, drop_zeros=True)
    assert K.nnz - Kd.nnz == ref["exact_zero_entries"] or K.nnz - Kd.nnz <= ref["exact_zero_entries"]


@pytest.fixture(scope="module")
def mesh6():
    return box_tet_mesh(6, seed=3)


def test_stiffness_properties(mesh6):
    K = O.stiffnessMatrix(mesh6)
    assert abs(K - K.T).max() == 0.0
    assert np.abs(K.sum(axis=1)).max() < 1e-13 * np.abs(K.data).max() * 20
    M = O.massMatrix(mesh6)
    assert abs(M.sum() - 1000.0) < 1e-9        # total volume of [-5,5]^3
    u = 2 * mesh6.p[0] + 3 * mesh6.p[1] - mesh6.p[2]
    free = mesh6.dirichlet_mask() == 0
    assert np.abs((K @ u)[free]).max() < 1e-12 * np.abs(K.data).max() * 10
    H = O.hfield(mesh6, u)
    assert np.allclose(H, np.array([[-2.0], [-3.0], [1.0]]), atol=1e-12)


def test_p2_patch_and_partition():
    m = box_tet_mesh(3, seed=1, order=2)
    K = O.quadraticStiffnessMatrix(m)
    q = m.p[0] ** 2 - m.p[1] * m.p[2]   # quadratic field: the nodal rule is not exact, so only linear
    u = 2 * m.p[0] - m.p[2]
    free = m.dirichlet_mask() == 0
    assert np.abs((K @ u)[free]).max() < 1e-10
    assert np.abs(K.sum(axis=1)).max() < 1e-12
    Mf = O.quadraticMassMatrix(m, full_phi=True)
    # weights sum to 1/6 and are scaled by VE (src/FEM3D.jl:535), so the total is V/6
    assert abs(Mf.sum() - 1000.0 / 6) < 1e-9
    del q


@pytest.mark.parametrize("full_phi", [True, False])
def test_p2_convection_known_answers(full_phi):
    """C[r, c] = int (u . grad phi_r) phi_c (the reference's scatter of Ck[j, i],
    src/FEM3D.jl:640-648): its columns sum to 0 (sum_r phi_r = 1) and, for a constant
    velocity and a linear T = a . x, (C^T T)_c = (u . a) int phi_c = (u . a) (M 1)_c.
    Both hold for the linear-part-only phi too, whose basis still sums to 1."""
    m = box_tet_mesh(3, seed=1, order=2)
    rng = np.random.default_rng(5)
    C = O.quadraticConvectionMatrix(m, rng.normal(size=(3, m.nv)), full_phi=full_phi)
    assert np.abs(np.asarray(C.sum(axis=0))).max() < 1e-12 * np.abs(C.data).max()
    uc = np.tile(np.array([[0.3], [-1.2], [0.7]]), m.nv)
    a = np.array([2.0, -1.0, 0.5])
    C = O.quadraticConvectionMatrix(m, uc, full_phi=full_phi)
    M = O.quadraticMassMatrix(m, full_phi=full_phi)
    lhs, rhs = C.T @ (a @ m.p), (uc[:, 0] @ a) * (M @ np.ones(m.nv))
    assert np.abs(lhs - rhs).max() < (1e-12 if full_phi else 1e-9) * np.abs(rhs).max()
    # the other orientation is not the reference's matrix
    assert np.abs(C @ (a @ m.p) - rhs).max() > 1e-3 * np.abs(rhs).max()


def test_tangent_zero_field_and_symmetry(mesh6):
    rng = np.random.default_rng(0)
    H = rng.normal(size=(3, mesh6.nt))
    H[:, 0] = 0.0
    dmu = -rng.uniform(1e-10, 1e-9, mesh6.nt)
    T = O.tangentialStiffnessMatrix(mesh6, H, dmu)
    assert np.isfinite(T.data).all()
    assert abs(T - T.T).max() == 0.0


def test_froehlich_derivative_fd():
    for h in (0.0, 10.0, 1e3, 8e4):
        mu, dmu = O.froehlich(h, 1.2e6, 500.0)
        eps = max(1e-3, h * 1e-6)
        fd = (O.froehlich(h + eps, 1.2e6, 500.0)[0] - O.froehlich(h - eps, 1.2e6, 500.0)[0]) / (2 * eps) \
            if h > 0 else (O.froehlich(eps, 1.2e6, 500.0)[0] - mu) / eps
        assert abs(fd - dmu) <= 1e-6 * abs(dmu) + (1e-9 * abs(dmu) if h > 0 else 2e-3 * abs(dmu))
        assert abs(mu - MU0 * (1 + 1.2e6 / (500.0 + h))) < 1e-20


def test_pcg_matches_direct(mesh6):
    A = (O.stiffnessMatrix(mesh6) + O.massMatrix(mesh6)).tocsc()
    b = np.random.default_rng(1).normal(size=mesh6.nv)
    x, it, rr = O.pcg(A, b, tol=1e-13)
    xd = spla.spsolve(A, b)
    assert it > 0 and rr <= 1e-13
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-10


def test_linear_magnetostatics_matches_direct():
    m = box_tet_mesh(8, seed=4)
    mu = np.where(m.elementID == 2, 1000 * MU0, MU0)
    u0 = -m.p[0].copy()
    u, H, it = O.linear_magnetostatics(m, u0, mu, cg_tol=1e-13)
    K = O.stiffnessMatrix(m, mu).tocsr()
    fx = m.dirichlet_mask().astype(bool)
    free = ~fx
    ud = u0.copy()
    ud[free] = spla.spsolve(K[free][:, free].tocsc(), -(K[free][:, fx] @ u0[fx]))
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-10


def newton_case(n=10, seed=2):
    m = box_tet_mesh(n, seed=seed)
    nl = (m.elementID == 2).astype(np.uint8)
    mu_lin = np.full(m.nt, MU0)
    u0 = -(np.array([8e4, 0, 0])[:, None] * m.p).sum(axis=0)
    return m, nl, mu_lin, u0


def test_newton_fixed_point_and_line_search_modes():
    m, nl, mu_lin, u0 = newton_case()
    sols = {}
    for ls in ("residual", "reference"):   # a full-step Newton does not converge on this plate
        u, H, mu, st = O.newton(m, u0, nl, mu_lin, 1.2e6, 500.0, cg_tol=1e-12, line_search=ls)
        assert st["converged"], (ls, st)
        sols[ls] = (u, H)
    # the converged potential solves F(u) = -K(mu(u)) u = 0 on free rows
    u, H = sols["residual"]
    h = np.sqrt((H * H).sum(axis=0))
    mu = np.where(nl == 1, MU0 * (1 + 1.2e6 / (500 + h)), mu_lin)
    F = -(O.stiffnessMatrix(m, mu) @ u)
    free = m.dirichlet_mask() == 0
    F0 = -(O.stiffnessMatrix(m, np.where(nl == 1, MU0 * (1 + 1.2e6 / (500 + 8e4)), mu_lin)) @ u0)
    assert np.linalg.norm(F[free]) < 1e-9 * np.linalg.norm(F0[free])
    for ls in ("reference",):
        assert np.linalg.norm(sols[ls][1] - H) / np.linalg.norm(H) < 1e-8


def test_adjoint_matches_finite_differences():
    m = box_tet_mesh(6, seed=9)
    rng = np.random.default_rng(5)
    mur = rng.uniform(1, 1000, m.nt)
    mu = mur * MU0
    c = m.centroids()
    target = (np.sqrt((c * c).sum(axis=0)) < 2.0).astype(np.uint8)
    u0 = -m.p[0].copy()
    u, H, it = O.linear_magnetostatics(m, u0, mu, cg_tol=1e-14)
    grad, lam = O.adjoint(m, target, mu, u, cg_tol=1e-14)
    for k in rng.choice(m.nt, 6, replace=False):
        d = 1e-6 * mur[k]
        vals = []
        for s in (+1, -1):
            mu2 = mu.copy()
            mu2[k] = (mur[k] + s * d) * MU0
            u2, _, _ = O.linear_magnetostatics(m, u0, mu2, cg_tol=1e-14)
            vals.append(O.objective_hx(m, target, u2))
        fd = (vals[0] - vals[1]) / (2 * d)
        an = grad[k] * MU0
        assert abs(fd - an) <= 1e-5 * abs(an) + 1e-12 * np.abs(grad * MU0).max()


def test_heat_be_matches_direct():
    m = box_tet_mesh(5, seed=6)
    kappa = np.exp(np.random.default_rng(3).normal(size=m.nt))
    T0 = np.exp(-((m.p ** 2).sum(axis=0)) / 0.5 ** 2)
    T, snaps, tot = O.heat_be(m, T0, kappa, 1.0, 1e-3, 10, cg_tol=1e-13, every=5)
    K = O.stiffnessMatrix(m, kappa)
    M = O.massMatrix(m)
    A = (M + 1e-3 * K).tocsr()
    fx = m.dirichlet_mask().astype(bool)
    free = ~fx
    Td = T0.copy()
    Td[fx] = 0
    for _ in range(10):
        b = M @ Td
        Td[free] = spla.spsolve(A[free][:, free].tocsc(), b[free])
    assert np.linalg.norm(T - Td) / np.linalg.norm(Td) < 1e-10
    assert snaps.shape == (2, m.nv)


def test_boundary_integral_and_lagrange():
    m = box_tet_mesh(4, seed=0)
    C = O.lagrange(m)
    assert abs(C.sum() - 1000.0) < 1e-9
    F = np.array([1.0, 2.0, 3.0])
    R = O.BoundaryIntegral(m, F)
    # closed surface: the flux of a constant field integrates to zero
    assert abs(R.sum()) < 1e-10
    # faces with normal +x carry +F_x A/3 per node
    assert abs(R[m.boundary_nodes].sum()) < 1e-10


def test_triangle_mesh_properties():
    m = box_tri_mesh(6, seed=2)
    K = O.stiffnessMatrix2D(m)
    assert np.abs(K.sum(axis=1)).max() < 1e-13
    assert abs(O.massMatrix2D(m).sum() - 100.0) < 1e-10
    m2 = box_tri_mesh(4, seed=2, order=2)
    assert abs(O.quadraticMassMatrix2D(m2).sum() - 100.0) < 1e-9
    u = 2 * m2.p[0] - 3 * m2.p[1]
    free = m2.dirichlet_mask() == 0
    assert np.abs((O.quadraticStiffnessMatrix2D(m2) @ u)[free]).max() < 1e-10


def test_demag_field_matches_direct_solve():
    """Micromagnetics/LL.jl:162-211 restated: PCG on the singular Neumann problem vs a
    direct solve with one node pinned (H does not see the constant)."""
    import scipy.sparse.linalg as spla
    m = box_tet_mesh(8, seed=3)
    rng = np.random.default_rng(0)
    M = rng.normal(size=(3, m.nv))
    M /= np.linalg.norm(M, axis=0)
    c = m.centroids()
    inside = (np.sqrt((c * c).sum(0)) < 3.0).astype(np.uint8)
    Hn, u, it = O.magnetostaticField(m, M, inside)
    K = O.stiffnessMatrix(m).tocsr()
    rhs = np.zeros(m.nv)
    for k in np.flatnonzero(inside):
        nds = m.t[:, k]
        f = M[:, nds].mean(axis=1)
        for a in range(4):
            r = O.abcd(m, k, a)
            rhs[nds[a]] += m.VE[k] * (r[1] * f[0] + r[2] * f[1] + r[3] * f[2])
    assert abs(rhs.sum()) < 1e-12
    ud = np.zeros(m.nv)
    ud[1:] = spla.spsolve(K[1:, 1:].tocsc(), rhs[1:])
    Hd = O.hfield(m, ud)
    Hnd, vol = np.zeros((3, m.nv)), np.zeros(m.nv)
    for k in np.flatnonzero(inside):
        for a in range(4):
            vol[m.t[a, k]] += m.VE[k]
            Hnd[:, m.t[a, k]] += m.VE[k] * Hd[:, k]
    with np.errstate(invalid="ignore", divide="ignore"):
        Hnd /= vol
    ok = np.isfinite(Hnd[0])
    assert np.array_equal(np.isfinite(Hn), np.isfinite(Hnd))
    assert np.linalg.norm(Hn[:, ok] - Hnd[:, ok]) / np.linalg.norm(Hnd[:, ok]) < 1e-10


def test_nedelec_known_answers():
    """Whitney edge elements (src/FEM3D.jl:155-191): every element block is symmetric
    and annihilates the edge values of a gradient, (phi_j - phi_i) / l_e in the local
    orientation; on one element, the edge values of A = B0 x x / 2 (midpoint rule,
    exact for a linear A) give B = curl A = B0 exactly, and the load vector is
    Ak-consistent: RHS = Ak u for that A."""
    rng = np.random.default_rng(3)
    m = box_tet_mesh(2, seed=5, order=2)
    Ak = O.nedelecLocalStiffness(m)
    I, J = [0, 1, 2, 3, 2, 1], [1, 2, 0, 0, 3, 3]
    for k in range(m.nt):
        blk = Ak[:, k].reshape(6, 6)
        assert np.abs(blk - blk.T).max() <= 1e-12 * np.abs(blk).max()
        v = m.t[:4, k]
        phi = rng.normal(size=4)
        le = np.linalg.norm(m.p[:, v[J]] - m.p[:, v[I]], axis=0)
        g = (phi[J] - phi[I]) / le
        assert np.abs(blk @ g).max() <= 1e-10 * np.abs(blk).max() * np.abs(g).max()
    # one element
    p = rng.normal(size=(3, 4))
    mids = [(0, 1), (1, 2), (2, 0), (3, 0), (3, 2), (3, 1)]
    P = np.hstack([p, np.stack([(p[:, a] + p[:, b]) / 2 for a, b in mids], axis=1)])
    t = np.arange(10, dtype=np.int32).reshape(10, 1)
    one = MESH(order=2, dim=3, p=P, t=t, surfaceT=np.zeros((4, 0), np.int32), elementID=np.ones(1, np.int32),
               InsideElements=np.zeros(0, np.int32), InsideNodes=np.zeros(0, np.int32),
               VE=element_volumes(P, t[:4]), AE=np.zeros(0), normal=np.zeros((3, 0)), shell_id=(1,),
               boundary_nodes=np.zeros(0, np.int64))
    edges, ne = O.nedelec_edges(one)
    assert ne == 6 and np.array_equal(edges[:, 0], np.arange(6))
    B0 = np.array([0.5, -0.2, 0.3])
    u = np.zeros(6)
    for e in range(6):
        xm = 0.5 * (p[:, I[e]] + p[:, J[e]])
        d = p[:, J[e]] - p[:, I[e]]
        u[e] = 0.5 * np.cross(B0, xm) @ d / np.linalg.norm(d)
    Bf, Bn = O.nedelec_bfield(one, u)
    assert np.allclose(Bf[:, 0], B0, rtol=0, atol=1e-12) and abs(Bn[0] - np.linalg.norm(B0)) < 1e-12
    rhs = O.nedelec_load(one, B0)
    assert np.allclose(O.nedelecLocalStiffness(one)[:, 0].reshape(6, 6) @ u, rhs, rtol=0, atol=1e-12 * np.abs(rhs).max())


def test_oracle_scalar_potential_patch_test():
    """magnetostatics() of the C++ reference (Neumann, no Dirichlet rows): with a
    uniform factor mu = 1 the discrete solution is u = -Hext.x + c exactly (P1 holds
    linear fields, and the boundary integral of a linear basis over a face is AE/3)."""
    m = box_tet_mesh(4, seed=3)
    Hext = np.array([0.7, -0.2, 0.4])
    u, it, rr = O.scalarPotential(m, np.ones(m.nt), Hext, 1, tol=1e-14)
    exact = -(Hext[:, None] * m.p).sum(axis=0)
    d = u - exact
    assert np.abs(d - d.mean()).max() < 1e-10 * np.abs(exact).max()


def test_nedelec_reference_orientation_null_space():
    """The reference orients each element's six edges locally (src/mesh.jl:603-630),
    so elements sharing an edge may disagree: its curl-curl matrix is not that of a
    conforming edge space.  With one orientation per edge (low to high vertex) the
    null space is the discrete gradients, (vertices - 1)-dimensional; with the
    reference's it is smaller and the gradients are not in it."""
    import scipy.linalg as la
    m = box_tet_mesh(3, seed=6, order=2)
    edges, ne = O.nedelec_edges(m)
    t = np.asarray(m.t[:4])
    loc = [(0, 1), (1, 2), (2, 0), (3, 0), (2, 3), (1, 3)]
    A = O.nedelecStiffness(m).toarray()
    Ak = O.nedelecLocalStiffness(m)
    S = np.array([np.where(t[a] < t[b], 1.0, -1.0) for a, b in loc])
    Akc = Ak * np.stack([S[i] * S[j] for i in range(6) for j in range(6)])
    Ac = O._ned_global(m, Akc, edges, ne).toarray()

    def nullity(M):
        w = la.eigvalsh(M)
        return int((np.abs(w) < 1e-10 * np.abs(w).max()).sum())

    nvert = int(t.max()) + 1
    assert nullity(Ac) == nvert - 1
    assert nullity(A) < nvert - 1
    # discrete gradient oriented by each edge's first use, scaled by 1/length (the
    # edge unknowns are mean tangential components: curl N_e = 2 l_e grad l_i x grad l_j)
    G = np.zeros((ne, m.nv))
    seen = np.zeros(ne, dtype=bool)
    for k in range(m.nt):
        for le, (a, b) in enumerate(loc):
            e = edges[le, k]
            if not seen[e]:
                seen[e] = True
                ia, ib = t[a, k], t[b, k]
                ln = np.linalg.norm(m.p[:, ib] - m.p[:, ia])
                G[e, ib], G[e, ia] = 1.0 / ln, -1.0 / ln
    Gc = np.zeros((ne, m.nv))
    for k in range(m.nt):
        for le, (a, b) in enumerate(loc):
            e = edges[le, k]
            lo, hi = sorted((t[a, k], t[b, k]))
            ln = np.linalg.norm(m.p[:, hi] - m.p[:, lo])
            Gc[e] = 0.0
            Gc[e, hi], Gc[e, lo] = 1.0 / ln, -1.0 / ln
    assert np.abs(Ac @ Gc).max() <= 1e-10 * np.abs(Ac).max()
    assert np.abs(A @ G).max() > 0.1 * np.abs(A).max()
