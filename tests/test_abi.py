"""The C-ABI library builds, loads, and exports every entry point include/sphx/sphx.h declares."""
import ctypes
import os
import re

from sphinxsys_gb300 import build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sphx", "sphx.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sphx_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_declared_symbols():
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert set(declared_symbols()) == set(native.SIGNATURES)


def test_load_binds_signatures_without_a_device():
    lib = native.load()
    assert lib.sphx_version().decode().startswith("sphx-gb300")
    # host-only entry points work without a GPU
    md = native.MeshDesc()
    lo = (ctypes.c_double * 3)(-0.1, -0.1, 0)
    up = (ctypes.c_double * 3)(5.466, 5.466, 0)
    native.call("sphx_mesh_from_bounds", 2, lo, up, 0.065, 2, ctypes.byref(md))
    assert md.all_cells[0] == 90 and md.all_cells[1] == 90
    s = ctypes.c_double()
    native.call("sphx_lattice_number_density", 2, 0.0325, 0.025, ctypes.byref(s))
    assert abs(s.value - 1616.7570433713393) < 1e-9


def test_errors_are_returned_not_fatal():
    lib = native.load()
    st = lib.sphx_mesh_from_bounds(4, None, None, 0.1, 2, None)
    assert st == 1
    assert b"invalid" in lib.sphx_last_error()


def test_checked_build_builds_and_reports_itself():
    """The bounds-checked build (-DSPHX_CHECK) compiles, exports the same entry points and
    reports itself; the default build does not."""
    path = build.build(checked=True)
    assert path != build.LIB
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.sphx_checked_build() == 1
    assert native.load().sphx_checked_build() == 0
