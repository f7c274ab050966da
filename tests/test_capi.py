"""CPU tests of the C ABI: the library builds, loads, and exports exactly the
entry points the public header declares (no compute calls without a GPU)."""
import ctypes
import os
import re

from odil_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(odil_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_functions():
    names = header_functions()
    assert "odil_wave_loss_grad_f32" in names
    assert "odil_version" in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(built_lib):
    assert sorted(_capi.SIGNATURES) == header_functions()


def test_version_and_status_strings(built_lib):
    lib = _capi.load()
    assert lib.odil_version() >= 100
    assert lib.odil_status_string(0) == b"ok"
    assert b"workspace" in lib.odil_status_string(-7)
    assert lib.odil_status_string(-99) == b"unknown status"


def test_shape_errors_without_gpu(built_lib):
    """Argument validation happens on the host, before any launch."""
    lib = _capi.load()
    p = _capi.OdilWaveParams()
    p.nt, p.nx, p.dt, p.dx, p.c = 0, 4, 0.1, 0.1, 1.0
    st = lib.odil_wave_residual_f64(ctypes.byref(p), None, None, None)
    assert st == -1  # ODIL_ERR_SHAPE
    p.nt = 4
    p.dt = -1.0
    assert lib.odil_wave_residual_f64(ctypes.byref(p), None, None, None) == -8
    p.dt = 0.1
    assert lib.odil_wave_residual_f64(ctypes.byref(p), None, None, None) == -8
    p.nx = 4096
    assert lib.odil_wave_march_f64(ctypes.byref(p), ctypes.c_void_p(16),
                                   ctypes.c_void_p(16), None) == -1
    assert lib.odil_wave_workspace_bytes(ctypes.byref(p)) > 256


def test_boundary_table_size_and_refusals_without_gpu(built_lib):
    """The boundary table of a solve from zero holds rows 0 and 1 in full
    and columns 0 and nx-1 of every further row; the table march refuses,
    on the host, grids where one lane would hold both edge columns."""
    lib = _capi.load()
    p = _capi.OdilWaveParams()
    p.dt, p.dx, p.c = 0.1, 0.1, 1.0
    for nt, nx in ((1, 5), (2, 5), (3, 1), (7, 2), (1024, 1024), (300, 777)):
        p.nt, p.nx = nt, nx
        want = min(nt, 2) * nx + max(nt - 2, 0) * min(nx, 2)
        assert lib.odil_wave_boundary_cells(ctypes.byref(p)) == want
    p.nt, p.nx = 0, 4
    assert lib.odil_wave_boundary_cells(ctypes.byref(p)) == 0
    p.nt, p.nx = 16, 4  # nx <= cpt 4: refused before anything launches
    st = lib.odil_wave_march_tiled_table_f32(
        ctypes.byref(p), ctypes.c_void_p(256), ctypes.c_void_p(256), 4, 48,
        16, 1, 0, None)
    assert st == -1  # ODIL_ERR_SHAPE
