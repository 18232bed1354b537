"""GPU: a plan is refused on a device other than the one it was created on.

A plan's window and twiddle tables live on its creation device; a kernel
launched while another device is current would read them through addresses of
the wrong device.  Every compute entry point checks the current device first
and returns EFF_ERR_INVALID before it queues a memset or a launch.  With one
GPU the mismatch is staged by overwriting the plan's recorded device through
the testing hook; the buffers passed are valid, so nothing faults even if a
check were missing, and the unchanged NaN outputs show that nothing ran.
"""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def test_mismatched_device_is_refused_before_any_work(cuda):
    from vmbd_gb300 import _lib, geometry, synth
    from vmbd_gb300.eff import EffPlan

    lib = _lib.load()
    wa = geometry.win2winaux((96, 96), (2, 2), 0.5)
    sf = (9, 9)
    plan = EffPlan(wa, sf, "valid", device=cuda)
    x = torch.from_numpy(synth.blob_edge_image(wa.sx, seed=1)).to(cuda)
    f = torch.from_numpy(synth.motion_psfs(wa.K, sf, seed=2)).to(cuda)
    fhat = plan.psf_spectrum(f)
    xhat = plan.image_spectrum(x)
    y_obs = plan.forward_image(x, fhat)
    torch.cuda.synchronize(cuda)
    nan = float("nan")
    y = torch.full(plan.sy, nan, device=cuda)
    gx = torch.full(plan.sx, nan, device=cuda)
    gf = torch.full((plan.K,) + sf, nan, device=cuda)
    loss = torch.full((1,), nan, dtype=torch.float64, device=cuda)
    spec = torch.full(plan.spectrum_shape, complex(nan, nan), dtype=torch.complex64, device=cuda)
    ws = torch.empty(lib.eff_loss_grad_workspace_bytes(plan._h, 1), dtype=torch.uint8, device=cuda)
    st = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    h = plan._h
    calls = {
        "eff_psf_spectrum": lambda: lib.eff_psf_spectrum(h, _p(f), _p(spec), 1, st),
        "eff_image_spectrum": lambda: lib.eff_image_spectrum(h, _p(x), _p(spec), 1, st),
        "eff_forward_image": lambda: lib.eff_forward_image(h, _p(x), _p(fhat), _p(y), None, 1, st),
        "eff_forward_psf": lambda: lib.eff_forward_psf(h, _p(f), _p(xhat), _p(y), None, 1, st),
        "eff_forward_both": lambda: lib.eff_forward_both(h, _p(x), _p(f), _p(y), None, None, 1, st),
        "eff_forward_residual": lambda: lib.eff_forward_residual(h, _p(x), _p(f), _p(y_obs), _p(y), None, None,
                                                                 1, st),
        "eff_adjoint": lambda: lib.eff_adjoint(h, _p(y_obs), _p(fhat), _p(xhat), _p(gx), _p(gf),
                                               _lib.ADJ_EXACT, 1, st),
        "eff_adjoint_residual": lambda: lib.eff_adjoint_residual(h, _p(y_obs), _p(y_obs), _p(fhat), _p(xhat),
                                                                 _p(gx), _p(gf), _p(loss), _lib.ADJ_EXACT, 1, st),
        "eff_deconv_xdirect": lambda: lib.eff_deconv_xdirect(h, _p(y_obs), _p(fhat), _p(xhat), _p(gx), _p(gf),
                                                             0.0, 0.01, 1, st),
        "eff_loss_grad": lambda: lib.eff_loss_grad(h, _p(x), _p(f), _p(y_obs), _p(loss), _p(gx), _p(gf), _p(ws),
                                                   ws.numel(), 1, st),
        "eff_loss_grad_static": lambda: lib.eff_loss_grad_static(h, _p(x), _p(f), _p(y_obs), _p(loss), _p(gx),
                                                                 _p(gf), 1, st),
    }
    assert lib.eff_test_plan_set_device(h, cuda.index + 1) == _lib.EFF_OK
    try:
        for name, call in calls.items():
            assert call() == _lib.EFF_ERR_INVALID, name
            assert b"device" in lib.eff_last_error(), name
        arr = (ctypes.c_void_p * 1)(h.value)
        counts = (ctypes.c_int * 1)(1)
        b = ctypes.c_void_p()
        assert lib.eff_batch_create(arr, counts, 1, ctypes.byref(b)) == _lib.EFF_ERR_INVALID
        assert b"device" in lib.eff_last_error()
        torch.cuda.synchronize(cuda)
        for t in (y, gx, gf, loss):
            assert torch.isnan(t).all()
        assert torch.isnan(spec.real).all()
    finally:
        assert lib.eff_test_plan_set_device(h, cuda.index) == _lib.EFF_OK
    # back on its own device the plan works again
    assert calls["eff_forward_image"]() == _lib.EFF_OK
    torch.cuda.synchronize(cuda)
    assert torch.isfinite(y).all()
