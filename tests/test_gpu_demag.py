"""GPU demagnetising field (fg_demag_field, Micromagnetics/LL.jl:162-211) against the
oracle restatement: nodal field within 1e-8, NaN on the same nodes."""
import numpy as np
import pytest

import femeko_gpu as fg
import oracle as O

pytestmark = pytest.mark.gpu


def demag_case(n=8, seed=3, radius=3.0):
    m = fg.box_tet_mesh(n, seed=seed)
    rng = np.random.default_rng(0)
    M = rng.normal(size=(3, m.nv))
    M /= np.linalg.norm(M, axis=0)
    c = m.centroids()
    inside = (np.sqrt((c * c).sum(0)) < radius).astype(np.uint8)
    return m, M, inside


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_demag_field_matches_oracle(precision):
    m, M, inside = demag_case()
    Hn, u, st = fg.magnetostaticField(m, M, inside, precision=precision, rtol=1e-12)
    Ho, uo, it = O.magnetostaticField(m, M, inside, cg_tol=1e-13)
    assert st["converged"]
    ok = np.isfinite(Ho[0])
    assert np.array_equal(np.isfinite(Hn), np.isfinite(Ho))
    assert np.linalg.norm(Hn[:, ok] - Ho[:, ok]) / np.linalg.norm(Ho[:, ok]) < 1e-8


def test_demag_operator_kept_across_steps():
    """Two magnetisation states on one handle (the operator is assembled once): each
    field matches its own oracle solve."""
    m, M, inside = demag_case(n=7)
    for s in range(2):
        Ms = np.roll(M, s, axis=1)
        Hn, _, st = fg.magnetostaticField(m, Ms, inside, rtol=1e-12)
        Ho, _, _ = O.magnetostaticField(m, Ms, inside, cg_tol=1e-13)
        ok = np.isfinite(Ho[0])
        assert np.linalg.norm(Hn[:, ok] - Ho[:, ok]) / np.linalg.norm(Ho[:, ok]) < 1e-8
