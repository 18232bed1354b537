"""GPU: the deterministic overlap-add mode (EffGeom.flags EFF_GEOM_DETERMINISTIC).

The kernels store each patch's output tile and a gather kernel sums the tiles
covering a pixel in a fixed order, as the reference's gather overlap-add does
(gputools.cu:276-314): repeated forwards, image adjoints, loss/gradient steps
and deconvolutions give bit-identical results.  The results still match the
FP64 oracle at the parity tolerance and the atomic mode to FP32 rounding.
"""
import numpy as np
import pytest

from oracle import eff64
from vmbd_gb300 import geometry, synth

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _case(sx, csf, sf, sw=None, hop=None, mode="valid", kind="motion", seed=0, batch=None):
    wa = geometry.win2winaux(sx, csf, 0.5, sw=sw, nhop=hop)
    g = eff64.Geometry(sx, sf, csf, wa.sw, wa.nhop, mode)
    gen = synth.gaussian_psfs if kind == "gauss" else synth.motion_psfs
    n = batch or 1
    x = np.stack([synth.blob_edge_image(sx, seed=seed + i) for i in range(n)])
    f = np.stack([gen(g.K, sf, seed=seed + 10 + i) for i in range(n)])
    rng = np.random.default_rng(seed + 20)
    y_obs = np.stack([(eff64.forward(x[i], f[i], g, wa.ws.astype(np.float64)) +
                       0.01 * rng.standard_normal(g.sy)).astype(np.float32) for i in range(n)])
    if batch is None:
        x, f, y_obs = x[0], f[0], y_obs[0]
    return wa, g, x, f, y_obs


CASES = {
    # 512x512, 8x8 grid of 96x96 patches, 31x31 motion PSFs (frame 128)
    "cfg2_literal": dict(sx=(512, 512), csf=(8, 8), sf=(31, 31), sw=(96, 96), hop=(48, 48)),
    # odd geometry, same mode, mixed-parity patches, frame 64
    "same_odd": dict(sx=(70, 90), csf=(3, 4), sf=(9, 7), mode="same", kind="gauss", seed=3),
    # the MFBD workload's geometry on frame 256
    "mfbd_winaux": dict(sx=(536, 536), csf=(8, 8), sf=(25, 25), seed=5),
}


@pytest.mark.parametrize("name", list(CASES))
def test_deterministic_outputs_repeat_bitwise(cuda, name):
    import torch
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, y_obs = _case(**CASES[name])
    det = EffPlan(wa, g.sf, g.mode, device=cuda, deterministic=True)
    ato = EffPlan(wa, g.sf, g.mode, device=cuda)
    xt, ft, yt = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, f, y_obs))
    ws = wa.ws.astype(np.float64)

    def run(plan):
        xh, fh = plan.empty_spectrum(), plan.empty_spectrum()
        y = plan.forward_both(xt, ft, xhat_out=xh, fhat_out=fh)
        r = plan.forward_both(xt, ft, subtract=yt)
        gx, gf = plan.adjoint(r, fh, xh)
        loss, gx2, gf2 = plan.loss_grad(xt, ft, yt)
        yi = plan.forward_image(xt, fh)
        out = [y, r, gx, gf, loss, gx2, gf2, yi]
        if g.mode != "full":
            u, fz = plan.deconv_xdirect(y, fhat=fh, xhat=xh, alpha=1e-2, beta=1e-2)
            out += [u, fz]
        torch.cuda.synchronize(cuda)
        return [o.detach().cpu().numpy().copy() for o in out]

    a = run(det)
    for _ in range(3):
        b = run(det)
        for i, (p, q) in enumerate(zip(a, b)):
            assert p.tobytes() == q.tobytes(), (name, i)
    c = run(ato)
    for i, (p, q) in enumerate(zip(a, c)):
        assert rel(p, q) < 1e-5, (name, i, rel(p, q))
    y_ref = eff64.forward(x, f, g, ws)
    assert rel(a[0], y_ref) < TOL
    assert rel(a[1], y_ref - y_obs) < TOL
    res = a[1].astype(np.float64)
    assert rel(a[2], eff64.adjoint_image(res, f, g, ws)) < TOL
    assert rel(a[3], eff64.adjoint_psf(res, x, g, ws)) < TOL
    assert abs(float(a[4]) - 0.5 * np.sum(res ** 2)) < 1e-5 * 0.5 * np.sum(res ** 2)
    assert det.device_errors() == 0


def test_deterministic_batch_equals_single_images(cuda):
    import torch
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, y_obs = _case(sx=(200, 232), csf=(3, 4), sf=(12, 10), mode="same", kind="gauss", seed=7, batch=2)
    det = EffPlan(wa, g.sf, g.mode, device=cuda, deterministic=True)
    xt, ft, yt = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, f, y_obs))
    loss, gx, gf = det.loss_grad(xt, ft, yt)
    torch.cuda.synchronize(cuda)
    for i in range(2):
        li, gxi, gfi = det.loss_grad(xt[i], ft[i], yt[i])
        torch.cuda.synchronize(cuda)
        assert float(li) == float(loss[i])
        assert np.array_equal(gxi.cpu().numpy(), gx[i].cpu().numpy())
        assert np.array_equal(gfi.cpu().numpy(), gf[i].cpu().numpy())


def test_deterministic_plan_rejected_by_persistent_batch(cuda):
    from vmbd_gb300 import _lib
    from vmbd_gb300.eff import EffBatch, EffPlan
    wa = geometry.win2winaux((96, 96), (2, 2), 0.5)
    det = EffPlan(wa, (9, 9), "valid", device=cuda, deterministic=True)
    with pytest.raises(_lib.EffError, match="deterministic"):
        EffBatch([det], [2])
