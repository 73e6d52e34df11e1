"""Mesh files in the reference's save2file text format (src/geometry.jl:237-245,
src/mesh.jl:233-242): reader, writer and the GPU path on a loaded mesh.

tests/golden/saved_mesh_tet1/ is a hand-written one-tetrahedron folder in the text
Julia's join(row, " , ") produces for these arrays (1-based Int32 indices, Float64
shortest forms such as 0.16666666666666666 and -0.0).
"""
import os

import numpy as np
import pytest

import femeko_gpu as fg

HERE = os.path.dirname(os.path.abspath(__file__))
TET1 = os.path.join(HERE, "golden", "saved_mesh_tet1")


def test_fixture_parses():
    m = fg.load_mesh(TET1)
    assert m.dim == 3 and m.order == 1 and m.nv == 4 and m.nt == 1 and m.ns == 4
    assert np.array_equal(m.p, np.array([[0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], dtype=float))
    assert np.array_equal(m.t[:, 0], [0, 1, 2, 3])
    assert m.VE[0] == 1.0 / 6.0
    assert np.array_equal(m.surfaceT[:3, 0], [0, 2, 1]) and np.all(m.surfaceT[3] == 1)
    assert np.signbit(m.normal[0, 0]) and m.normal[0, 0] == 0.0
    assert m.AE[3] == np.sqrt(3.0) / 2.0
    assert np.array_equal(m.boundary_nodes, [0, 1, 2, 3])
    assert np.array_equal(m.elementID, [2]) and np.array_equal(m.InsideElements, [0])


@pytest.mark.parametrize("kind", ["tet", "tet10", "tri"])
def test_round_trip(tmp_path, kind):
    m = {"tet": lambda: fg.box_tet_mesh(3, seed=2), "tet10": lambda: fg.box_tet_mesh(2, seed=3, order=2),
         "tri": lambda: fg.box_tri_mesh(4, seed=1)}[kind]()
    fg.save_mesh(str(tmp_path), m)
    r = fg.load_mesh(str(tmp_path))
    assert r.dim == m.dim and r.order == m.order
    for name in ("p", "t", "surfaceT", "VE", "AE", "normal", "InsideElements", "InsideNodes", "boundary_nodes",
                 "elementID"):
        a, b = np.asarray(getattr(m, name)), np.asarray(getattr(r, name))
        assert a.shape == b.shape and np.array_equal(a, b), name
        if a.dtype.kind == "f":
            assert np.array_equal(np.signbit(a), np.signbit(b)), name


def test_save2file_text(tmp_path):
    f = str(tmp_path / "a.txt")
    fg.save2file(f, np.array([[1, 2, 3], [4, 5, 6]], dtype=np.int32))
    assert open(f).read() == "1 , 2 , 3\n4 , 5 , 6\n"
    fg.save2file(f, np.array([0.5, -0.0, 1e-5]))
    assert open(f).read().splitlines() == ["0.5", "-0.0", "1e-05"]
    v = fg.load2array(f)
    assert v[2] == 1e-5 and np.signbit(v[1])


def test_bad_files_are_rejected(tmp_path):
    fg.save_mesh(str(tmp_path), fg.box_tet_mesh(2, seed=1))
    with open(tmp_path / "t.txt", "a") as f:
        f.write("1 , 2\n")
    with pytest.raises(ValueError):
        fg.load_mesh(str(tmp_path))
    fg.save_mesh(str(tmp_path), fg.box_tet_mesh(2, seed=1))
    t = fg.load2array(str(tmp_path / "t.txt"), np.int64)
    t[0, 0] = 10 ** 6
    fg.save2file(str(tmp_path / "t.txt"), t)
    with pytest.raises(ValueError):
        fg.load_mesh(str(tmp_path))


@pytest.mark.gpu
def test_loaded_mesh_on_the_gpu(tmp_path):
    """A mesh read back from the files assembles bit-identically and solves the same
    linear magnetostatic problem."""
    m = fg.box_tet_mesh(6, seed=4)
    fg.save_mesh(str(tmp_path), m)
    r = fg.load_mesh(str(tmp_path))
    mu = np.where(m.elementID == 2, 1000 * fg.MU0, fg.MU0)
    Ka, Kb = fg.stiffnessMatrix(m, mu), fg.stiffnessMatrix(r, mu)
    assert np.array_equal(Ka.indptr, Kb.indptr) and np.array_equal(Ka.indices, Kb.indices)
    assert np.array_equal(Ka.data.view(np.uint64), Kb.data.view(np.uint64))
    u0 = -m.p[0].copy()
    ua, Ha, sa = fg.magnetostatics_linear(m, mu, u0)
    ub, Hb, sb = fg.magnetostatics_linear(r, mu, u0)
    assert np.array_equal(Ha.view(np.uint64), Hb.view(np.uint64))
