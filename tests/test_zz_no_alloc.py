"""GPU: eff_loss_grad_static, the loss/gradient step for callers that cannot
allocate device memory or pass a workspace (a binding of the reference's
objective/gradient interface hands over only data and outputs).

Called through the C ABI twice in a row -- the second call runs on whatever
the first left in the library's static scratch array -- and checked against
the workspace-taking eff_loss_grad within the tolerance of the other parity
tests.  Kept in a file of its own that collects last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _two_calls_match_workspace_step(lib, plan, x, f, y_obs, batch, cuda):
    import torch
    from vmbd_gb300 import _lib

    assert lib.eff_loss_grad_workspace_bytes(plan._h, batch) <= lib.eff_static_scratch_bytes()
    ref_loss, ref_gx, ref_gf = plan.loss_grad(x, f, y_obs)
    lead = (batch,) if batch > 1 else ()
    loss = torch.empty(batch, dtype=torch.float64, device=cuda)
    gx = torch.empty(lead + plan.sx, device=cuda)
    gf = torch.empty(lead + (plan.K,) + plan.sf, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    for _ in range(2):
        for t in (loss, gx, gf):
            t.fill_(float("nan"))
        status = lib.eff_loss_grad_static(plan._h, _p(x), _p(f), _p(y_obs), _p(loss), _p(gx), _p(gf),
                                          batch, stream)
        assert status == _lib.EFF_OK, lib.eff_last_error()
        torch.cuda.synchronize(cuda)
        assert rel(gx, ref_gx) < TOL
        assert rel(gf, ref_gf) < TOL
        ref = ref_loss.reshape(-1).double().cpu()
        assert (loss.cpu() - ref).abs().max().item() <= TOL * ref.abs().max().item()


def test_static_scratch_step_matches_workspace_step(cuda):
    import torch
    from vmbd_gb300 import _lib, geometry, synth
    from vmbd_gb300.eff import EffPlan

    lib = _lib.load()
    # 512x512 image, 8x8 grid of 96x96 patches, 31x31 motion PSFs
    wa = geometry.win2winaux((512, 512), (8, 8), 0.5, sw=(96, 96), nhop=(48, 48))
    sf = (31, 31)
    plan = EffPlan(wa, sf, "valid", device=cuda)
    x = torch.from_numpy(synth.blob_edge_image((512, 512), seed=5)).to(cuda)
    f = torch.from_numpy(synth.motion_psfs(wa.K, sf, seed=6)).to(cuda)
    gen = torch.Generator(device=cuda).manual_seed(7)
    y_obs = plan.forward_both(x, f) + 0.01 * torch.randn(plan.sy, device=cuda, generator=gen)
    _two_calls_match_workspace_step(lib, plan, x, f, y_obs, 1, cuda)


def test_static_scratch_step_batch_of_two(cuda):
    # two 256x256 images (4x4 grid of 64x64 patches, 15x15 PSFs) in one call:
    # the scratch holds the workspace layout at its batched, padded size
    import torch
    from vmbd_gb300 import _lib, geometry, synth
    from vmbd_gb300.eff import EffPlan

    lib = _lib.load()
    wa = geometry.win2winaux((256, 256), (4, 4), 0.5, sw=(64, 64), nhop=(32, 32))
    sf = (15, 15)
    plan = EffPlan(wa, sf, "valid", device=cuda)
    x = torch.stack([torch.from_numpy(synth.blob_edge_image((256, 256), seed=s)) for s in (21, 22)]).to(cuda)
    f = torch.stack([torch.from_numpy(synth.gaussian_psfs(wa.K, sf, seed=s)) for s in (23, 24)]).to(cuda)
    gen = torch.Generator(device=cuda).manual_seed(25)
    y_obs = plan.forward_both(x, f) + 0.01 * torch.randn((2,) + plan.sy, device=cuda, generator=gen)
    _two_calls_match_workspace_step(lib, plan, x, f, y_obs, 2, cuda)


def test_static_scratch_rejects_oversized_work(cuda):
    from vmbd_gb300 import _lib, geometry
    from vmbd_gb300.eff import EffPlan

    lib = _lib.load()
    wa = geometry.win2winaux((512, 512), (8, 8), 0.5, sw=(96, 96), nhop=(48, 48))
    plan = EffPlan(wa, (31, 31), "valid", device=cuda)
    batch = 1
    while lib.eff_loss_grad_workspace_bytes(plan._h, batch) <= lib.eff_static_scratch_bytes():
        batch += 1
    # rejected on the host before any pointer is used or any work is queued
    status = lib.eff_loss_grad_static(plan._h, ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
                                      None, ctypes.c_void_p(16), None, batch, None)
    assert status == _lib.EFF_ERR_UNSUPPORTED
    assert b"static" in lib.eff_last_error()
