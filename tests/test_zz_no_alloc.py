"""fg_cg_csc_noalloc (device-pointer CG that allocates nothing) against fg_cg_csc.

Collected last on purpose (file name): it must pass both alone and after the rest of
the GPU suite has used the library on the same device.
"""
import ctypes as C

import numpy as np
import pytest

import femeko_gpu as fg
import femeko_gpu._lib as L
import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _system(seed):
    mesh = fg.box_tet_mesh(6, seed=5)
    K = (O.stiffnessMatrix(mesh) + O.massMatrix(mesh)).tocsc()
    K.sort_indices()
    b = np.random.default_rng(seed).normal(size=mesh.nv)
    return K, b


def _noalloc(K, b, x0=None, rtol=1e-10):
    dev = torch.device("cuda", torch.cuda.current_device())
    colptr = torch.tensor(K.indptr.astype(np.int64), device=dev)
    rowval = torch.tensor(K.indices.astype(np.int64), device=dev)
    nzval = torch.tensor(K.data, dtype=torch.float64, device=dev)
    bd = torch.tensor(b, dtype=torch.float64, device=dev)
    xd = torch.zeros(K.shape[0], dtype=torch.float64, device=dev) if x0 is None else \
        torch.tensor(x0, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    o = fg.solve_opts(precision="fp64", rtol=rtol)
    s = L.SolveStats()
    st = L.lib().fg_cg_csc_noalloc(K.shape[0], colptr.data_ptr(), rowval.data_ptr(), nzval.data_ptr(), 0,
                                   bd.data_ptr(), xd.data_ptr(), C.byref(o), None, C.byref(s))
    L.check(st)
    return xd.cpu().numpy(), L.stats_dict(s)


def test_noalloc_matches_cg_csc_twice():
    K, b = _system(8)
    x_ref = fg.cg(K, b, reltol=1e-10, precision="fp64")
    for _ in range(2):   # two calls in a row share the scratch
        x, st = _noalloc(K, b)
        assert st["converged"]
        assert np.linalg.norm(K @ x - b) / np.linalg.norm(b) < 1.5e-10
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-8


def test_noalloc_second_system_no_leftover_state():
    K, b1 = _system(1)
    _, b2 = _system(2)
    x1, _ = _noalloc(K, b1)
    x2, _ = _noalloc(K, b2)
    r2 = fg.cg(K, b2, reltol=1e-10, precision="fp64")
    assert np.linalg.norm(x2 - r2) / np.linalg.norm(r2) < 1e-8
    assert np.linalg.norm(x1 - x2) > 0


def test_noalloc_rejects_oversize_and_host_pointers():
    lib = L.lib()
    o = fg.solve_opts(precision="fp64")
    s = L.SolveStats()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = dummy.data_ptr()
    st = lib.fg_cg_csc_noalloc(131072 + 1, p, p, p, 0, p, p, C.byref(o), None, C.byref(s))
    assert st == L.FG_BAD_ARG and b"exceed" in lib.fg_last_error()
    K, b = _system(3)
    host = np.zeros(K.shape[0])
    st = lib.fg_cg_csc_noalloc(K.shape[0], L.ptr(K.indptr.astype(np.int64)), L.ptr(K.indices.astype(np.int64)),
                               L.ptr(K.data), 0, L.ptr(b), L.ptr(host), C.byref(o), None, C.byref(s))
    assert st == L.FG_BAD_ARG and b"device" in lib.fg_last_error()
