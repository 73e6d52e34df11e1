"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports every
function include/femeko_gpu.h declares.  No compute call (no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?(?:void|fg_status|int32_t|int64_t|char|int|double)\s*\**\s*(\w+)\s*\(",
                             src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def libfg():
    import femeko_gpu._lib as L
    return L.lib()


def test_header_declares_functions():
    names = declared_functions()
    assert "fg_mesh_create" in names and "fg_newton_magnetostatics" in names
    # the reference's own ccall entry point, exported under its own name
    assert "scalarPotential" in names
    assert len(names) >= 15


def test_library_exports_all_declared(libfg):
    missing = [n for n in declared_functions() if not hasattr(libfg, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    import femeko_gpu._lib as L
    covered = set(L.SIGNATURES) | set(L.VOID_FUNCS) | {"fg_last_error", "fg_version", "fg_kernel_launches"}
    assert set(declared_functions()) <= covered


def test_version_and_error_string(libfg):
    assert libfg.fg_version() >= 1
    assert isinstance(libfg.fg_last_error(), bytes)


def test_build_targets_sm103a():
    import importlib.util
    spec = importlib.util.spec_from_file_location("b", os.path.join(ROOT, "femeko.jl_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert mod.ARCH == "-gencode=arch=compute_103a,code=sm_103a"
