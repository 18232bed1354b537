"""ctypes binding of ``libvmbd_eff.so`` (the C ABI in include/vmbd_eff.h).

The library is built in tree by ``vmbd_gb300.build``.  Loading fails loudly:
there is no CPU fallback for any operation of this package.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

EFF_OK = 0
EFF_ERR_INVALID = 1
EFF_ERR_UNSUPPORTED = 2
EFF_ERR_CUDA = 3

MODES = {"valid": 0, "same": 1, "full": 2}
ADJ_EXACT = 0
ADJ_REFERENCE = 1
OUT_ZEROED = 1
LOSS_OF_Y = 2
AFTER_FORWARD = 4
OPERAND_IMAGE = 0
OPERAND_PSF = 1
GEOM_DETERMINISTIC = 1
PROJ_CLIP_NORMALIZE = 0
PROJ_SIMPLEX = 1

# Every symbol include/vmbd_eff.h declares.
EXPORTS = (
    "eff_plan_create", "eff_plan_destroy", "eff_plan_frame", "eff_spectrum_bytes",
    "eff_psf_spectrum", "eff_image_spectrum", "eff_forward_image", "eff_forward_psf",
    "eff_adjoint", "eff_project_psf", "eff_basis_project", "eff_last_error",
    "eff_forward_both", "eff_adjoint_residual", "eff_loss_grad_workspace_bytes", "eff_loss_grad",
    "eff_static_scratch_bytes", "eff_loss_grad_static", "eff_edgetaper",
    "eff_adjoint_masked", "eff_dots3", "eff_pg_step", "eff_mu_update", "eff_max_nonneg",
    "eff_set_cluster_mode", "eff_batch_create", "eff_batch_destroy", "eff_batch_items",
    "eff_batch_forward_both", "eff_batch_adjoint_residual", "eff_deconv_xdirect", "eff_forward_ex",
    "eff_adjoint_ex", "eff_forward_residual", "eff_batch_forward_residual", "eff_test_plan_set_device",
    "eff_forward_both_ex", "eff_plan_device_errors", "eff_set_spectrum_staging", "eff_set_image_tile",
)


class EffGeom(ctypes.Structure):
    _fields_ = [("sx", ctypes.c_int * 2), ("sf", ctypes.c_int * 2), ("csf", ctypes.c_int * 2),
                ("sw", ctypes.c_int * 2), ("hop", ctypes.c_int * 2), ("sfft", ctypes.c_int),
                ("mode", ctypes.c_int), ("threads", ctypes.c_int), ("flags", ctypes.c_int)]


class EffError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"vmbd_eff error {code}: {msg}")
        self.code = code


_LIB = None
_DEBUG_LIB = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the library (building it first when it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError(f"{_build.LIB} is missing: run vmbd_gb300.build.build()")
    _LIB = _bind(ctypes.CDLL(_build.LIB))
    return _LIB


def load_debug(build_if_missing: bool = True) -> ctypes.CDLL:
    """The bounds-checked variant (frames 64 and 128; see vmbd_gb300.build):
    the same C ABI, for tests that run small cases through it and then read
    the plan's device error word."""
    global _DEBUG_LIB
    if _DEBUG_LIB is not None:
        return _DEBUG_LIB
    if build_if_missing and not _build.up_to_date(debug=True):
        _build.build(debug=True)
    if not os.path.exists(_build.DEBUG_LIB):
        raise RuntimeError(f"{_build.DEBUG_LIB} is missing: run vmbd_gb300.build.build(debug=True)")
    _DEBUG_LIB = _bind(ctypes.CDLL(_build.DEBUG_LIB))
    return _DEBUG_LIB


def _bind(L: ctypes.CDLL) -> ctypes.CDLL:
    """Set the argument and result types of every exported entry point."""
    vp, ip, fp = ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p
    sig = {
        "eff_plan_create": ([ctypes.POINTER(EffGeom), fp, fp, ctypes.POINTER(vp)], ip),
        "eff_plan_destroy": ([vp], ip),
        "eff_plan_frame": ([vp, ctypes.POINTER(ctypes.c_int)], ip),
        "eff_spectrum_bytes": ([vp], ctypes.c_size_t),
        "eff_psf_spectrum": ([vp, fp, vp, ip, vp], ip),
        "eff_image_spectrum": ([vp, fp, vp, ip, vp], ip),
        "eff_forward_image": ([vp, fp, vp, fp, vp, ip, vp], ip),
        "eff_forward_psf": ([vp, fp, vp, fp, vp, ip, vp], ip),
        "eff_adjoint": ([vp, fp, vp, vp, fp, fp, ip, ip, vp], ip),
        "eff_project_psf": ([fp, ip, ip, ip, vp], ip),
        "eff_basis_project": ([fp, fp, fp, ip, ip, vp], ip),
        "eff_last_error": ([], ctypes.c_char_p),
        "eff_forward_both": ([vp, fp, fp, fp, vp, vp, ip, vp], ip),
        "eff_forward_residual": ([vp, fp, fp, fp, fp, vp, vp, ip, vp], ip),
        "eff_adjoint_residual": ([vp, fp, fp, vp, vp, fp, fp, vp, ip, ip, vp], ip),
        "eff_loss_grad_workspace_bytes": ([vp, ip], ctypes.c_size_t),
        "eff_loss_grad": ([vp, fp, fp, fp, vp, fp, fp, vp, ctypes.c_size_t, ip, vp], ip),
        "eff_static_scratch_bytes": ([], ctypes.c_size_t),
        "eff_edgetaper": ([fp, ip, ip, fp, ip, fp, ip, ip, vp], ip),
        "eff_adjoint_masked": ([vp, fp, fp, vp, vp, fp, fp, ip, ip, vp], ip),
        "eff_dots3": ([fp, fp, ctypes.c_longlong, fp, fp, ctypes.c_longlong, vp, ip, vp], ip),
        "eff_pg_step": ([fp, fp, fp, fp, ip, ip, vp, ip, fp, fp, ctypes.c_longlong, vp], ip),
        "eff_max_nonneg": ([fp, ctypes.c_longlong, vp, vp], ip),
        "eff_set_cluster_mode": ([ip], ip),
        "eff_test_plan_set_device": ([vp, ip], ip),
        "eff_plan_device_errors": ([vp, ctypes.POINTER(ctypes.c_int), ip], ip),
        "eff_set_spectrum_staging": ([ip], ip),
        "eff_set_image_tile": ([ip], ip),
        "eff_batch_create": ([vp, vp, ip, ctypes.POINTER(vp)], ip),
        "eff_batch_destroy": ([vp], ip),
        "eff_batch_items": ([vp], ip),
        "eff_batch_forward_both": ([vp, vp, vp, vp, vp, vp, vp], ip),
        "eff_batch_forward_residual": ([vp, vp, vp, vp, vp, vp, vp, vp], ip),
        "eff_batch_adjoint_residual": ([vp, vp, vp, vp, vp, vp, vp, vp, vp], ip),
        "eff_mu_update": ([fp, fp, fp, ctypes.c_float, ip, ip, ip, ip, vp, ctypes.c_float, vp, ip, fp,
                           ctypes.c_longlong, vp], ip),
        "eff_forward_ex": ([vp, ip, fp, vp, fp, fp, vp, ip, fp, ctypes.c_longlong, vp, ip, ip, vp], ip),
        "eff_adjoint_ex": ([vp, fp, fp, fp, vp, vp, fp, fp, vp, ip, ip, ip, vp], ip),
        "eff_forward_both_ex": ([vp, fp, fp, fp, fp, vp, vp, ip, fp, ctypes.c_longlong, vp, ip, ip, vp], ip),
        "eff_loss_grad_static": ([vp, fp, fp, fp, vp, fp, fp, ip, vp], ip),
        "eff_deconv_xdirect": ([vp, fp, vp, vp, fp, fp, ctypes.c_float, ctypes.c_float, ip, vp], ip),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


def check(status: int, lib=None) -> None:
    """Raise EffError for a non-OK status with the message of the library the
    call went to (default the product library)."""
    if status != EFF_OK:
        msg = (lib or load()).eff_last_error().decode(errors="replace")
        raise EffError(status, msg)
