"""ctypes binding of libfemeko_gpu.so (the C ABI declared in include/femeko_gpu.h).

There is no CPU fallback: every call goes to the CUDA library, and loading fails
loudly when the library is missing and cannot be built.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "libfemeko_gpu.so")

FG_OK, FG_NOT_CONVERGED, FG_NAN, FG_BAD_ARG, FG_BAD_MESH, FG_CUDA, FG_NO_DEVICE, FG_UNSUPPORTED = range(8)
STATUS_NAMES = {0: "FG_OK", 1: "FG_NOT_CONVERGED", 2: "FG_NAN", 3: "FG_BAD_ARG", 4: "FG_BAD_MESH", 5: "FG_CUDA",
                6: "FG_NO_DEVICE", 7: "FG_UNSUPPORTED"}
FG_FP64, FG_MIXED = 0, 1
FG_LS_NONE, FG_LS_REFERENCE, FG_LS_RESIDUAL, FG_LS_QUADRATIC = 0, 1, 2, 3


class FemekoGPUError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class SolveOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("rtol", C.c_double), ("maxiter", C.c_int32), ("inner_rtol", C.c_double),
                ("check_every", C.c_int32), ("use_graph", C.c_int32), ("spmv", C.c_int32),
                ("reserved_", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("converged", C.c_int32), ("pad_", C.c_int32),
                ("relres", C.c_double), ("ms", C.c_double)]


class NewtonOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("maxit", C.c_int32), ("tol_update", C.c_double),
                ("inner_rtol", C.c_double), ("cg_maxiter", C.c_int32), ("line_search", C.c_int32),
                ("min_step", C.c_double), ("Ms", C.c_double), ("Hk", C.c_double), ("check_every", C.c_int32),
                ("use_graph", C.c_int32), ("forcing", C.c_int32), ("picard_steps", C.c_int32), ("eta_min", C.c_double),
                ("eta_max", C.c_double)]


class NewtonStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int32), ("cg_iters", C.c_int32), ("converged", C.c_int32),
                ("trials", C.c_int32), ("update_ratio", C.c_double), ("residual", C.c_double),
                ("alpha", C.c_double), ("energy", C.c_double), ("ms", C.c_double), ("setup_ms", C.c_double),
                ("cg_ms", C.c_double)]


class AdjointStats(C.Structure):
    _fields_ = [("forward_iters", C.c_int32), ("adjoint_iters", C.c_int32), ("newton_iters", C.c_int32),
                ("converged", C.c_int32), ("forward_ms", C.c_double), ("adjoint_ms", C.c_double)]


class BatchStats(C.Structure):
    _fields_ = [("problems", C.c_int32), ("converged", C.c_int32), ("max_iterations", C.c_int32),
                ("cluster_ctas", C.c_int32), ("total_iterations", C.c_int64), ("ms", C.c_double),
                ("max_refinements", C.c_int32), ("reserved_", C.c_int32)]


def stats_dict(s) -> dict:
    return {name: getattr(s, name) for name, _ in s._fields_ if name != "pad_"}


_vp = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int32
_d = C.c_double

# name -> argtypes; every function returns fg_status (int)
SIGNATURES = {
    "fg_device_info": [C.c_char_p, _i32, C.POINTER(_i32)],
    "fg_mesh_create": [_vp, _i64, _vp, _i64, _i32, _i32, C.POINTER(_vp)],
    "fg_mesh_destroy": [_vp],
    "fg_mesh_nnz": [_vp, C.POINTER(_i64), C.POINTER(_i32)],
    "fg_mesh_set_dirichlet": [_vp, _vp],
    "fg_mesh_volumes": [_vp, _vp],
    "fg_csc_pattern": [_vp, _vp, _vp, _i32],
    "fg_stiffness": [_vp, _vp, _vp],
    "fg_mass": [_vp, _vp, _i32, _vp],
    "fg_tangent": [_vp, _vp, _vp, _vp],
    "fg_convection": [_vp, _vp, _vp, _i32, _vp],
    "fg_local_stiffness": [_vp, _vp, _vp],
    "fg_lagrange": [_vp, _vp],
    "fg_boundary_integral": [_vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _i32, _vp],
    "fg_cg_csc": [_i64, _vp, _vp, _vp, _i32, _vp, _vp, C.POINTER(SolveOpts), C.POINTER(SolveStats)],
    "fg_spmv_csc": [_i64, _vp, _vp, _vp, _i32, _vp, _vp],
    "fg_cg_csc_noalloc": [_i64, _vp, _vp, _vp, _i32, _vp, _vp, C.POINTER(SolveOpts), _vp, C.POINTER(SolveStats)],
    "fg_magnetostatics_linear": [_vp, _vp, _vp, C.POINTER(SolveOpts), _vp, _vp, C.POINTER(SolveStats)],
    "fg_newton_magnetostatics": [_vp, _vp, _vp, _vp, C.POINTER(NewtonOpts), _vp, _vp, _vp, C.POINTER(NewtonStats)],
    "fg_hfield": [_vp, _vp, _vp],
    "fg_demag_field": [_vp, _vp, _vp, C.POINTER(SolveOpts), _vp, _vp, C.POINTER(SolveStats)],
    "fg_newton_set_inputs": [_vp, _vp, _vp, _vp],
    "fg_newton_solve_resident": [_vp, C.POINTER(NewtonOpts), C.POINTER(NewtonStats)],
    "fg_newton_get_outputs": [_vp, _vp, _vp, _vp],
    "fg_heat_be": [_vp, _vp, _d, _d, _i32, _vp, _i32, _vp, C.POINTER(SolveOpts), C.POINTER(SolveStats)],
    "fg_boundary_mass": [_vp, _vp, _vp, _vp, _i64, _vp],
    "fg_edge_mesh_create": [_vp, _i64, _vp, _vp, _i64, _i64, _i32, C.POINTER(_vp)],
    "fg_nedelec_local_stiffness": [_vp, _vp],
    "fg_nedelec_stiffness": [_vp, _vp, _vp],
    "fg_nedelec_tangent": [_vp, _vp, _vp, _vp, _vp],
    "fg_nedelec_load": [_vp, _vp, _vp],
    "fg_nedelec_bfield": [_vp, _vp, _vp, _vp],
    "fg_nedelec_linear": [_vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(SolveOpts), C.POINTER(SolveStats)],
    "fg_nedelec_newton": [_vp, _vp, _vp, _vp, _vp, _vp, _i32, _d, _i32, _d, _vp, _vp, _vp, _vp, _vp,
                          C.POINTER(SolveOpts), C.POINTER(SolveStats)],
    "fg_transport_be": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _d, _i32, _i32, _vp, _i32, _vp,
                        C.POINTER(SolveOpts), C.POINTER(SolveStats)],
    "fg_batch_magnetostatics_linear": [_vp, _i32, _vp, _vp, C.POINTER(SolveOpts), _vp, _vp, C.POINTER(BatchStats)],
    "fg_magnetostatics_sweep": [_vp, _vp, _i32, _vp, C.POINTER(SolveOpts), _vp, C.POINTER(SolveStats)],
    "fg_adjoint_dJdmu": [_vp, _vp, _vp, _vp, _vp, C.POINTER(NewtonOpts), _d, C.POINTER(_d), _vp, _vp,
                         C.POINTER(AdjointStats)],
    "fg_scalar_potential_newton": [_vp, _i64, _vp, _i64, _i32, _vp, _vp, _vp, _vp, C.POINTER(NewtonOpts), _vp, _vp,
                                   _vp, C.POINTER(NewtonStats)],
    "fg_scalar_potential": [_vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _i32, C.POINTER(SolveOpts),
                            C.POINTER(SolveStats)],
    "fg_scalar_potential_status": [],
    "fg_bench_kernel": [_vp, _i32, _i32, _i32, C.POINTER(_d)],
    "fg_mesh_layout": [_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i32)],
    "fg_autotune": [_vp, _i32, C.POINTER(_i32), _vp, _i32],
    "fg_set_cg_variant": [_vp, _i32, _i32],
    "fg_get_cg_variant": [_vp, _i32, C.POINTER(_i32)],
}
VOID_FUNCS = {"fg_solve_opts_default": [C.POINTER(SolveOpts)], "fg_newton_opts_default": [C.POINTER(NewtonOpts)],
              # the reference's own void entry point (Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:49-61)
              "scalarPotential": [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int]}

_lib = None


def lib():
    """Load the library (building it in-tree with nvcc when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        import importlib.util
        spec = importlib.util.spec_from_file_location("femeko_gpu_build", os.path.join(PKG_ROOT, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = C.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    for name, args in VOID_FUNCS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = None
    L.fg_last_error.restype = C.c_char_p
    L.fg_last_error.argtypes = []
    L.fg_version.restype = C.c_int32
    L.fg_kernel_launches.restype = C.c_int64
    L.fg_kernel_launches.argtypes = []
    _lib = L
    return L


def check(status: int, allow_not_converged: bool = False) -> int:
    if status == FG_OK or (allow_not_converged and status == FG_NOT_CONVERGED):
        return status
    raise FemekoGPUError(status, lib().fg_last_error().decode(errors="replace"))


def ptr(a):
    """Data pointer of a numpy array; the returned object keeps the array alive for the
    duration of the call (temporaries created inside a call expression stay valid)."""
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# Handles still open at interpreter exit are released before the CUDA runtime tears
# itself down (a cudaFree issued after that point is undefined).
import weakref  # noqa: E402

_open_handles = weakref.WeakSet()
_shutting_down = False


def register_handle(obj):
    _open_handles.add(obj)


def unregister_handle(obj):
    _open_handles.discard(obj)


def _close_all():
    global _shutting_down
    for obj in list(_open_handles):
        try:
            obj.close()
        except Exception:
            pass
    _shutting_down = True


import atexit  # noqa: E402

atexit.register(_close_all)
