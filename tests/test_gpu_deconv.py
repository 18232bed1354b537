"""GPU: Fourier-division deconvolution (OlaGPU.deconv 'xdirect' / 'direct',
olaGPU.py:515-609) through the C ABI, against the reference's golden vectors
and the FP64 oracle.

Tolerance: relative L2 <= 1e-5 (FP32 kernels vs FP64 oracle / FP32
reference) for image estimates.  PSF estimates divide by |X-hat|^2, whose
dynamic range (~1e9) turns FP32 FFT rounding into errors of a few 1e-5 in any
FP32 pipeline: they are held to max(1e-5, 3 x the error of the oracle's FP32
restatement, ``eff64.deconv_xdirect_fp32``) against the same reference."""
import glob
import os

import numpy as np
import pytest

from oracle import eff64
from vmbd_gb300 import geometry, synth

pytestmark = pytest.mark.gpu
TOL = 1e-5
DECONV_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_deconv_*.npz")))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def psf_tol(y, x, g, ws, alpha, beta, ref):
    """max(TOL, 3x the all-FP32 restatement's error against ``ref``)."""
    e32 = rel(eff64.deconv_xdirect_fp32(y, x, g, ws, "psf", alpha, beta), ref)
    return max(TOL, 3.0 * e32)


def t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)


@pytest.mark.parametrize("path", DECONV_GOLDEN, ids=lambda p: os.path.basename(p))
def test_xdirect_matches_reference_golden(cuda, path):
    from vmbd_gb300 import OlaGPU
    z = np.load(path)
    c = {k: z[k] for k in z.files}
    mode = str(c["mode"])
    wa = geometry.Winaux(tuple(c["sx"]), tuple(c["csf"]), tuple(c["sw"]), tuple(c["hop"]))
    alpha, beta = float(c["alpha"]), float(c["beta"])
    F = OlaGPU(c["f"], tuple(c["sx"]), mode, wa)
    X = OlaGPU(c["x"], tuple(c["sf"]), mode, wa)
    u = F.deconv(c["y"], mode="xdirect", alpha=alpha, beta=beta)
    fz = X.deconv(c["y"], mode="xdirect", alpha=alpha, beta=beta)
    assert isinstance(u, np.ndarray) and u.shape == tuple(c["sx"])
    assert fz.shape == c["fz"].shape
    assert rel(u, c["u"]) < TOL
    g = eff64.Geometry(tuple(c["sx"]), tuple(c["sf"]), tuple(c["csf"]), tuple(c["sw"]), tuple(c["hop"]), mode,
                       tuple(c["sfft"]))
    assert rel(fz, c["fz"]) < psf_tol(c["y"], c["x"], g, c["ws"].astype(np.float64), alpha, beta, c["fz"])


# geometry, mode, alpha, beta, forced plan frame for the object (0: auto)
CASES = {
    # 512^2, 8x8 grid of 96^2 patches, 31^2 motion PSFs (frame 128)
    "cfg2_literal": (dict(sx=(512, 512), csf=(8, 8), sf=(31, 31), sw=(96, 96), hop=(48, 48), kind="motion"),
                     "valid", 0.0, 1e-2, 0),
    # win2winaux geometry of the MFBD frames (E 144, frame 256)
    "cfg3_winaux": (dict(sx=(536, 536), csf=(8, 8), sf=(25, 25), kind="motion"), "valid", 1e-2, 1e-3, 0),
    # objects on the 192 frame: the division runs on a second plan at the
    # reference's 256 frame
    "cfg3_winaux_obj192": (dict(sx=(536, 536), csf=(8, 8), sf=(25, 25), kind="motion"), "valid", 1e-2, 1e-3, 192),
    "same_laplacian": (dict(sx=(200, 232), csf=(3, 4), sf=(12, 10)), "same", 5e-2, 1e-3, 0),
}


def make(sx, csf, sf, sw=None, hop=None, kind="gauss", seed=0, mode="valid"):
    wa = geometry.win2winaux(sx, csf, 0.5, sw=sw, nhop=hop)
    x = synth.blob_edge_image(sx, seed=seed)
    gen = synth.gaussian_psfs if kind == "gauss" else synth.motion_psfs
    f = gen(wa.K, sf, seed=seed + 1)
    E = [wa.sw[d] + sf[d] - 1 for d in range(2)]
    ref = tuple(1 << int(np.ceil(np.log2(e))) for e in E)
    g = eff64.Geometry(sx, sf, csf, wa.sw, wa.nhop, mode, ref)
    ws = wa.ws.astype(np.float64)
    y = eff64.forward(x, f, g, ws)
    y = y + 0.01 * np.random.default_rng(seed + 2).standard_normal(y.shape)
    return wa, g, ws, x, f, y.astype(np.float32)


@pytest.mark.parametrize("name", list(CASES))
def test_xdirect_matches_fp64_oracle(cuda, name):
    from vmbd_gb300 import OlaGPU
    spec, mode, alpha, beta, sfft = CASES[name]
    wa, g, ws, x, f, y = make(**spec, mode=mode)
    F = OlaGPU(t(f, cuda), wa.sx, mode, wa, sfft=sfft)
    X = OlaGPU(t(x, cuda), g.sf, mode, wa, sfft=sfft)
    if sfft:
        assert F.plan.N == sfft and F._deconv_plan()[0].N == g.sfft[0]
    u = F.deconv(t(y, cuda), mode="xdirect", alpha=alpha, beta=beta).cpu().numpy()
    fz = X.deconv(t(y, cuda), mode="xdirect", alpha=alpha, beta=beta).cpu().numpy()
    u_ref = eff64.deconv_xdirect(y, eff64.psf_spectrum(f, g), g, ws, "image", alpha, beta)
    fz_ref = eff64.deconv_xdirect(y, eff64.image_spectrum(x, g, ws), g, ws, "psf", alpha, beta)
    assert rel(u, u_ref) < TOL, name
    assert rel(fz, fz_ref) < psf_tol(y, x, g, ws, alpha, beta, fz_ref), name


def test_xdirect_plan_level_batch_and_both_outputs(cuda):
    """Both outputs from one transform of y, batched images, against single
    calls."""
    import torch
    from vmbd_gb300.eff import EffPlan
    wa, g, ws, x, f, y = make(sx=(256, 256), csf=(4, 4), sf=(15, 15), sw=(64, 64), hop=(32, 32))
    plan = EffPlan(wa, g.sf, "valid", sfft=g.sfft[0], device=cuda)
    xs = torch.stack([t(x, cuda), t(np.flipud(x).copy(), cuda)])
    fs = torch.stack([t(f, cuda), t(f[::-1].copy(), cuda)])
    ys = torch.stack([t(y, cuda), t(np.fliplr(y).copy(), cuda)])
    fh = plan.psf_spectrum(fs)
    xh = plan.image_spectrum(xs)
    u, fz = plan.deconv_xdirect(ys, fhat=fh, xhat=xh, alpha=1e-2, beta=1e-2)
    for b in range(2):
        u1, _ = plan.deconv_xdirect(ys[b], fhat=fh[b], alpha=1e-2, beta=1e-2)
        _, f1 = plan.deconv_xdirect(ys[b], xhat=xh[b], alpha=1e-2, beta=1e-2)
        assert rel(u[b].cpu(), u1.cpu()) < 1e-6
        assert rel(fz[b].cpu(), f1.cpu()) < 1e-6
        u_ref = eff64.deconv_xdirect(ys[b].cpu().numpy(), eff64.psf_spectrum(fs[b].cpu().numpy(), g), g, ws,
                                     "image", 1e-2, 1e-2)
        assert rel(u[b].cpu(), u_ref) < TOL
    # no wait in the kernels ran out (the row hand-off between the cluster's
    # CTAs counts the bytes each single-output call sends)
    assert plan.device_errors() == 0


@pytest.mark.parametrize("cluster", [1, 2], ids=["cta", "cluster2"])
def test_xdirect_cluster_modes_agree(cuda, cluster):
    from vmbd_gb300 import _lib
    from vmbd_gb300.eff import EffPlan
    lib = _lib.load()
    wa, g, ws, x, f, y = make(**CASES["cfg2_literal"][0])
    plan = EffPlan(wa, g.sf, "valid", device=cuda)
    _lib.check(lib.eff_set_cluster_mode(cluster))
    try:
        u, fz = plan.deconv_xdirect(t(y, cuda), fhat=plan.psf_spectrum(t(f, cuda)),
                                    xhat=plan.image_spectrum(t(x, cuda)), alpha=0.0, beta=1e-2)
    finally:
        _lib.check(lib.eff_set_cluster_mode(0))
    assert rel(u.cpu(), eff64.deconv_xdirect(y, eff64.psf_spectrum(f, g), g, ws, "image", 0.0, 1e-2)) < TOL
    fz_ref = eff64.deconv_xdirect(y, eff64.image_spectrum(x, g, ws), g, ws, "psf", 0.0, 1e-2)
    assert rel(fz.cpu(), fz_ref) < psf_tol(y, x, g, ws, 0.0, 1e-2, fz_ref)
    assert plan.device_errors() == 0


def test_direct_mode_matches_oracle(cuda):
    from vmbd_gb300 import OlaGPU
    wa, g, ws, x, f, y = make(sx=(256, 256), csf=(4, 4), sf=(15, 15), kind="gauss", seed=5)
    F = OlaGPU(f, wa.sx, "valid", wa)
    u = F.deconv(y, mode="direct", alpha=1e-2, beta=1e-2)
    u_ref = eff64.deconv_direct(y, eff64.psf_spectrum(f, g), g, ws, 1e-2, 1e-2)
    assert u.shape == tuple(wa.sx)
    assert rel(u, u_ref) < TOL


def test_deconv_error_behaviour(cuda):
    from vmbd_gb300 import OlaGPU
    wa, g, ws, x, f, y = make(sx=(96, 96), csf=(2, 2), sf=(9, 9))
    F = OlaGPU(f, wa.sx, "valid", wa)
    X = OlaGPU(x, g.sf, "valid", wa)
    with pytest.raises(IOError):
        F.deconv(np.zeros((10, 10), np.float32), mode="xdirect")
    with pytest.raises(NotImplementedError):
        F.deconv(y, mode="sparse")
    with pytest.raises(NotImplementedError):
        X.deconv(y, mode="direct")
    Ffull = OlaGPU(f, wa.sx, "full", wa)
    with pytest.raises(NotImplementedError):
        Ffull.deconv(np.zeros(Ffull.sy, np.float32), mode="xdirect")
