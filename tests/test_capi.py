"""CPU: the C-ABI library builds for sm_103a, loads, and exports every entry
point include/vmbd_eff.h declares (no compute calls without a GPU)."""
import ctypes
import os
import re

from vmbd_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            src = open(os.path.join(ROOT, "include", name)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            syms |= set(re.findall(r"\b(eff_\w+)\s*\(", src))
    return syms


def test_header_declares_the_abi():
    syms = declared_symbols()
    assert {"eff_plan_create", "eff_forward_image", "eff_adjoint", "eff_project_psf"} <= syms
    assert syms == set(_lib.EXPORTS)


def test_library_builds_and_exports_every_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_loader_binds_every_symbol():
    L = _lib.load()
    for s in _lib.EXPORTS:
        assert getattr(L, s).restype is not None or s == "eff_plan_destroy"


def test_plan_rejects_bad_geometry_without_gpu():
    # argument checks run before any CUDA call
    L = _lib.load()
    g = _lib.EffGeom()
    g.sx[:] = (64, 64)
    g.sf[:] = (80, 80)  # PSF larger than image
    g.csf[:] = (2, 2)
    g.sw[:] = (32, 32)
    g.hop[:] = (16, 16)
    w = (ctypes.c_float * 128)()
    h = ctypes.c_void_p()
    assert L.eff_plan_create(ctypes.byref(g), w, w, ctypes.byref(h)) == _lib.EFF_ERR_INVALID
    assert b"PSF" in L.eff_last_error()
    g.sf[:] = (9, 9)
    g.mode = 7
    assert L.eff_plan_create(ctypes.byref(g), w, w, ctypes.byref(h)) == _lib.EFF_ERR_INVALID
    g.mode = 0
    g.sfft = 96  # not a supported frame edge
    assert L.eff_plan_create(ctypes.byref(g), w, w, ctypes.byref(h)) == _lib.EFF_ERR_UNSUPPORTED
    g.sfft = 0
    for bad in (100, 1024, -32):  # CTA size: a multiple of 32 up to the compiled maximum
        g.threads = bad
        assert L.eff_plan_create(ctypes.byref(g), w, w, ctypes.byref(h)) == _lib.EFF_ERR_INVALID
        assert b"threads" in L.eff_last_error()
    g.threads = 0
    assert L.eff_plan_create(None, w, w, ctypes.byref(h)) == _lib.EFF_ERR_INVALID


def test_compute_entry_points_reject_null_plan():
    L = _lib.load()
    assert L.eff_forward_image(None, None, None, None, None, 1, None) == _lib.EFF_ERR_INVALID
    assert L.eff_adjoint(None, None, None, None, None, None, 0, 1, None) == _lib.EFF_ERR_INVALID
    assert L.eff_project_psf(None, 1, 1, 0, None) == _lib.EFF_ERR_INVALID
    assert L.eff_spectrum_bytes(None) == 0


def test_adjoint_ex_flags_validate_without_gpu():
    # flag checks run before any CUDA call
    L = _lib.load()
    dummy = ctypes.c_void_p(16)
    assert L.eff_adjoint_ex(None, dummy, dummy, None, dummy, None, dummy, None, dummy, _lib.ADJ_EXACT,
                            _lib.LOSS_OF_Y, 1, None) == _lib.EFF_ERR_INVALID
    assert b"LOSS_OF_Y" in L.eff_last_error()
    assert L.eff_adjoint_ex(None, dummy, None, None, dummy, None, dummy, None, dummy, _lib.ADJ_EXACT,
                            0, 1, None) == _lib.EFF_ERR_INVALID
    assert b"y_obs" in L.eff_last_error()
    assert L.eff_adjoint_ex(None, dummy, None, None, dummy, None, dummy, None, dummy, _lib.ADJ_EXACT,
                            8, 1, None) == _lib.EFF_ERR_INVALID
    assert L.eff_forward_residual(None, dummy, dummy, dummy, dummy, None, None, 1, None) == _lib.EFF_ERR_INVALID
    assert L.eff_forward_residual(None, None, None, None, None, None, None, 1, None) == _lib.EFF_ERR_INVALID


def test_debug_library_exports_every_symbol():
    # the bounds-checked variant has the same C ABI
    path = build.build(debug=True)
    lib = ctypes.CDLL(path)
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert _lib.load_debug() is not _lib.load()
