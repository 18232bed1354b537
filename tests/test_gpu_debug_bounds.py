"""GPU: the bounds-checked build on the small parity fixtures.

The library's debug variant (``-DEFF_DEBUG``, frames 64 and 128) checks every
frame, shared-memory and global index its kernels form against the buffer it
addresses; a bad index is recorded in the plan's device error word and the
access skipped instead of made.  Every small reference fixture (odd and
non-square patches, mixed parity, same mode, a patch grid that does not cover
the image, the deconvolution cases) runs through it -- one CTA per patch and
2-CTA clusters, atomic and deterministic overlap-add, cached spectra from
global memory and staged in shared memory -- and must match the reference and
leave the error word clear.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import fixtures  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-5
SMALL = [p for p in fixtures.operator_paths() if not os.path.basename(p).startswith("ref_cfg")]


def rel(a, b, mask=None):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def dlib(cuda):
    from vmbd_gb300 import _lib
    return _lib.load_debug()


@pytest.mark.parametrize("det", [False, True], ids=["atomic", "deterministic"])
@pytest.mark.parametrize("cl,staging", [(1, 0), (2, 0), (2, 1)], ids=["cta", "cluster2", "cluster2-staged"])
@pytest.mark.parametrize("path", SMALL, ids=lambda p: os.path.basename(p))
def test_operator_fixtures_in_bounds(cuda, dlib, path, cl, staging, det):
    import torch
    from vmbd_gb300 import _lib, geometry
    from vmbd_gb300.eff import EffPlan
    c = fixtures.load(path)
    wa = geometry.Winaux(tuple(c["sx"]), tuple(c["csf"]), tuple(c["sw"]), tuple(c["hop"]))
    _lib.check(dlib.eff_set_cluster_mode(cl))
    _lib.check(dlib.eff_set_spectrum_staging(staging))
    try:
        plan = EffPlan(wa, tuple(c["sf"]), c["mode"], device=cuda, lib=dlib, deterministic=det)
        assert plan.N in (64, 128)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(cuda)  # noqa: E731
        x, f, r = t(c["x"]), t(c["f"]), t(c["r"])
        fh, xh = plan.psf_spectrum(f), plan.image_spectrum(x)
        y = plan.forward_image(x, fh).cpu().numpy()
        yb = plan.forward_both(x, f).cpu().numpy()
        yp = plan.forward_psf(f, xh).cpu().numpy()
        gx, gf = plan.adjoint(r, fh, xh, adjoint="reference")
        m = np.isfinite(c["y"])
        for out in (y, yb, yp):
            assert rel(out, c["y"], m) < TOL
        mx = np.isfinite(c["gx"])
        assert rel(gx.cpu().numpy(), c["gx"], mx) < TOL
        assert rel(gf.cpu().numpy(), c["gf"]) < TOL
        y_obs = t(np.where(m, c["y"], 0.0) + c["r"])
        loss, gx2, gf2 = plan.loss_grad(x, f, y_obs)
        assert np.isfinite(float(loss)) and torch.isfinite(gx2).all() and torch.isfinite(gf2).all()
        assert plan.device_errors() == 0
    finally:
        _lib.check(dlib.eff_set_cluster_mode(0))
        _lib.check(dlib.eff_set_spectrum_staging(2))  # the default


@pytest.mark.parametrize("path", fixtures.deconv_paths(), ids=lambda p: os.path.basename(p))
def test_deconv_fixtures_in_bounds(cuda, dlib, path):
    import torch
    from vmbd_gb300 import geometry
    from vmbd_gb300.eff import EffPlan
    c = fixtures.load(path)
    wa = geometry.Winaux(tuple(c["sx"]), tuple(c["csf"]), tuple(c["sw"]), tuple(c["hop"]))
    plan = EffPlan(wa, tuple(c["sf"]), c["mode"], sfft=int(np.max(c["sfft"])), device=cuda, lib=dlib)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(cuda)  # noqa: E731
    fh, xh = plan.psf_spectrum(t(c["f"])), plan.image_spectrum(t(c["x"]))
    u, fz = plan.deconv_xdirect(t(c["y"]), fhat=fh, xhat=xh, alpha=float(c["alpha"]), beta=float(c["beta"]))
    assert rel(u.cpu().numpy(), c["u"]) < TOL
    assert rel(fz.cpu().numpy(), c["fz"]) < 1e-4
    assert plan.device_errors() == 0
