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


def _device_system(K, b, x0=None, rowval=None):
    dev = torch.device("cuda", torch.cuda.current_device())
    d = dict(colptr=torch.tensor(K.indptr.astype(np.int64), device=dev),
             rowval=torch.tensor((K.indices if rowval is None else rowval).astype(np.int64), device=dev),
             nzval=torch.tensor(K.data, dtype=torch.float64, device=dev),
             b=torch.tensor(b, dtype=torch.float64, device=dev),
             x=torch.zeros(K.shape[0], dtype=torch.float64, device=dev) if x0 is None else
             torch.tensor(x0, dtype=torch.float64, device=dev))
    torch.cuda.synchronize()
    return d


def _call(n, d, rtol=1e-10, maxiter=1_000_000):
    o = fg.solve_opts(precision="fp64", rtol=rtol, maxiter=maxiter)
    s = L.SolveStats()
    st = L.lib().fg_cg_csc_noalloc(n, d["colptr"].data_ptr(), d["rowval"].data_ptr(), d["nzval"].data_ptr(), 0,
                                   d["b"].data_ptr(), d["x"].data_ptr(), C.byref(o), None, C.byref(s))
    return st, L.stats_dict(s)


def _noalloc(K, b, x0=None, rtol=1e-10):
    d = _device_system(K, b, x0)
    st, stats = _call(K.shape[0], d, rtol=rtol)
    L.check(st)
    return d["x"].cpu().numpy(), stats


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


def test_noalloc_allocates_nothing():
    """A warm call leaves the device's free memory and torch's allocator untouched."""
    K, b = _system(4)
    d = _device_system(K, b)
    st, _ = _call(K.shape[0], d)          # first call: scratch address looked up
    assert st == L.FG_OK
    d["x"].zero_()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
    st, stats = _call(K.shape[0], d)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    alloc1 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
    assert st == L.FG_OK and stats["converged"]
    assert free1 == free0 and alloc1 == alloc0


def test_noalloc_iteration_cap_and_default_cap():
    K, b = _system(5)
    d = _device_system(K, b)
    st, stats = _call(K.shape[0], d, maxiter=2)
    assert st == L.FG_NOT_CONVERGED and stats["iterations"] == 2 and not stats["converged"]
    d["x"].zero_()
    st, stats = _call(K.shape[0], d, maxiter=0)    # <= 0: the default cap, as with no options
    assert st == L.FG_OK and stats["converged"]


def test_noalloc_rejects_bad_structure_and_zero_diagonal():
    """Row indices outside the matrix and a zero diagonal are found on the device
    (every index is checked before it is used) and returned as FG_BAD_ARG."""
    lib = L.lib()
    K, b = _system(6)
    bad = K.indices.astype(np.int64).copy()
    bad[len(bad) // 2] = K.shape[0] + 5
    d = _device_system(K, b, rowval=bad)
    st, _ = _call(K.shape[0], d)
    assert st == L.FG_BAD_ARG and b"CSC" in lib.fg_last_error()
    Kz = K.copy()
    Kz.setdiag(Kz.diagonal())           # the diagonal is stored, then one entry set to 0
    Kz = Kz.tocsc()
    Kz.sort_indices()
    i = K.shape[0] // 3
    for k in range(Kz.indptr[i], Kz.indptr[i + 1]):
        if Kz.indices[k] == i:
            Kz.data[k] = 0.0
    d = _device_system(Kz, b)
    st, _ = _call(K.shape[0], d)
    assert st == L.FG_BAD_ARG and b"diagonal" in lib.fg_last_error()
    # a valid call afterwards runs normally (the control words are cleared per call)
    x, stats = _noalloc(K, b)
    assert stats["converged"]


@pytest.mark.skipif(not torch.cuda.is_available() or torch.cuda.device_count() < 2,
                    reason="needs memory of a second device")
def test_noalloc_rejects_other_device_memory():
    K, b = _system(7)
    d = _device_system(K, b)
    d["x"] = torch.zeros(K.shape[0], dtype=torch.float64, device="cuda:1")
    with torch.cuda.device(0):
        st, _ = _call(K.shape[0], d)
    assert st == L.FG_BAD_ARG
