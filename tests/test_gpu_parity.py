"""GPU parity of the fused EFF kernels (through the C ABI) against the
reference's golden vectors and the FP64 oracle.

Tolerance: relative L2 <= 1e-5 (FP32 kernels vs FP64 oracle), the bound the
operator's results are stated at.
"""
import os
import sys

import numpy as np
import pytest

from oracle import eff64
from vmbd_gb300 import geometry, synth

pytestmark = pytest.mark.gpu
TOL = 1e-5
sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import fixtures  # noqa: E402

# operator fixtures (cnv / cnvtp) and Fourier-division deconvolution fixtures
GOLDEN = fixtures.operator_paths()
DECONV_GOLDEN = fixtures.deconv_paths()


def rel(a, b, mask=None):
    cplx = np.iscomplexobj(a) or np.iscomplexobj(b)
    a = np.asarray(a, np.complex128 if cplx else np.float64)
    b = np.asarray(b, np.complex128 if cplx else np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)


def make(sx, csf, sf, sw=None, hop=None, mode="valid", kind="gauss", seed=0):
    wa = geometry.win2winaux(sx, csf, 0.5, sw=sw, nhop=hop)
    g = eff64.Geometry(sx, sf, csf, wa.sw, wa.nhop, mode)
    x = synth.blob_edge_image(sx, seed=seed)
    gen = synth.gaussian_psfs if kind == "gauss" else synth.motion_psfs
    f = gen(g.K, sf, seed=seed + 1)
    r = np.random.default_rng(seed + 2).standard_normal(g.sy).astype(np.float32)
    return wa, g, x, f, r


# ---------------------------------------------------------------------------
# golden vectors of the reference (OlaGPU run on its own kernels)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p))
def test_olagpu_matches_reference_golden(cuda, path):
    from vmbd_gb300 import OlaGPU
    c = fixtures.load(path)
    mode = c["mode"]
    wa = geometry.Winaux(tuple(c["sx"]), tuple(c["csf"]), tuple(c["sw"]), tuple(c["hop"]))
    F = OlaGPU(c["f"], tuple(c["sx"]), mode, wa, adjoint="reference")
    X = OlaGPU(c["x"], tuple(c["sf"]), mode, wa, adjoint="reference")
    y = F.cnv(c["x"])
    yX = X.cnv(c["f"])
    m = np.isfinite(c["y"])
    assert rel(y, c["y"], m) < TOL
    assert rel(yX, c["y"], m) < TOL
    assert np.all(y[~m] == 0)
    assert np.all(yX[~m] == 0)
    gx = F.cnvtp(c["r"])
    gf = X.cnvtp(c["r"])
    mx = np.isfinite(c["gx"])
    assert rel(gx, c["gx"], mx) < TOL
    assert rel(gf, c["gf"]) < TOL


# ---------------------------------------------------------------------------
# FP64 oracle, exact adjoints, at the workload geometries
# ---------------------------------------------------------------------------
CASES = {
    # 256^2, 4x4 grid of 64^2 patches, 15^2 Gaussian PSFs, frame 128
    "cfg1_literal": dict(sx=(256, 256), csf=(4, 4), sf=(15, 15), sw=(64, 64), hop=(32, 32)),
    "cfg1_winaux": dict(sx=(256, 256), csf=(4, 4), sf=(15, 15)),
    # 512^2, 8x8 grid of 96^2 patches, 31^2 motion PSFs, frame 128
    "cfg2_literal": dict(sx=(512, 512), csf=(8, 8), sf=(31, 31), sw=(96, 96), hop=(48, 48), kind="motion"),
    # 512^2, 8x8 winaux geometry (sw 122, E 152), frame 256
    "cfg2_winaux": dict(sx=(512, 512), csf=(8, 8), sf=(31, 31), kind="motion"),
    # the same geometry on the 192 frame (24 x 8 mixed radix)
    "cfg2_winaux_f192": dict(sx=(512, 512), csf=(8, 8), sf=(31, 31), kind="motion", sfft=192),
    # 512^2 frame of the MFBD workload, 25^2 PSFs, sw 120, frame 256
    "cfg3_winaux": dict(sx=(536, 536), csf=(8, 8), sf=(25, 25), kind="motion"),
    "cfg3_winaux_f192": dict(sx=(536, 536), csf=(8, 8), sf=(25, 25), kind="motion", sfft=192),
    # 384x512 member of the uneven batch: mixed-parity sw (116, 119), frame 256
    "cfg4_mixed": dict(sx=(404, 532), csf=(6, 8), sf=(21, 21), kind="motion"),
    "cfg4_mixed_f192": dict(sx=(404, 532), csf=(6, 8), sf=(21, 21), kind="motion", sfft=192),
    # a small geometry forced onto the 192 frame (zero padding well past E)
    "cfg1_literal_f192": dict(sx=(256, 256), csf=(4, 4), sf=(15, 15), sw=(64, 64), hop=(32, 32), sfft=192),
    "same_mode": dict(sx=(200, 232), csf=(3, 4), sf=(12, 10), mode="same"),
    "full_mode": dict(sx=(200, 232), csf=(3, 4), sf=(12, 10), mode="full"),
    # frame 512 (32 values per lane): extent 256 < E <= ~270 fits 4-CTA clusters at full
    # CTA size, larger extents (292, 424) run on 8-CTA clusters
    "frame512_cl4": dict(sx=(380, 380), csf=(2, 2), sf=(9, 9), sw=(262, 262), hop=(118, 118)),
    "frame512_cl8a": dict(sx=(400, 400), csf=(2, 2), sf=(25, 25), kind="motion"),
    "frame512_cl8": dict(sx=(600, 600), csf=(2, 2), sf=(25, 25), kind="motion"),
    "frame512_same": dict(sx=(400, 440), csf=(2, 2), sf=(25, 21), mode="same"),
    "full_mode_f192": dict(sx=(200, 232), csf=(3, 4), sf=(12, 10), mode="full", sfft=192),
    # frame 128 with odd extents (E 113 x 106: the cluster's CTAs own 58 and 56
    # rows of phase 3), an odd window height and a hop of 80 columns (the image
    # tile by the tensor engine: rows of 101-row windows, 96 of 336 columns)
    "tile_odd": dict(sx=(281, 336), csf=(3, 4), sf=(13, 11), sw=(101, 96), hop=(90, 80), kind="motion"),
    "tile_odd_same": dict(sx=(281, 336), csf=(3, 4), sf=(13, 11), sw=(101, 96), hop=(90, 80), kind="motion",
                          mode="same"),
    # frame 64 (extent 48 x 56): its CTAs have a spare warp for the DC column unit
    "frame64": dict(sx=(80, 96), csf=(3, 3), sf=(9, 9), kind="motion"),
    "frame64_same": dict(sx=(70, 90), csf=(3, 4), sf=(9, 7), mode="same"),
}
# frame each case runs on
FRAME = {"cfg1_literal": 128, "cfg1_winaux": 128, "cfg2_literal": 128, "cfg2_winaux": 256,
         "cfg2_winaux_f192": 192, "cfg3_winaux": 256, "cfg3_winaux_f192": 192, "cfg4_mixed": 256,
         "cfg4_mixed_f192": 192, "cfg1_literal_f192": 192, "frame512_cl4": 512, "frame512_cl8a": 512, "frame512_cl8": 512,
         "frame512_same": 512, "frame64": 64, "frame64_same": 64, "tile_odd": 128, "tile_odd_same": 128}


@pytest.fixture(params=[(1, 0), (2, 0), (2, 1)], ids=["cta", "cluster2", "cluster2-staged-spectra"])
def cluster_mode(request, cuda):
    """Run a test with one CTA per patch, then with a 2-CTA cluster; in the
    last run kernels that multiply by cached spectra stage them in shared
    memory by bulk copies (where they fit)."""
    from vmbd_gb300 import _lib
    lib = _lib.load()
    mode, staging = request.param
    _lib.check(lib.eff_set_cluster_mode(mode))
    _lib.check(lib.eff_set_spectrum_staging(staging))
    yield mode
    _lib.check(lib.eff_set_cluster_mode(0))
    _lib.check(lib.eff_set_spectrum_staging(2))  # the default


@pytest.mark.parametrize("name", list(CASES))
def test_operator_matches_fp64_oracle(cuda, cluster_mode, name):
    from vmbd_gb300.eff import EffPlan
    spec = dict(CASES[name])
    sfft = spec.pop("sfft", 0)
    wa, g, x, f, r = make(**spec)
    plan = EffPlan(wa, g.sf, g.mode, sfft=sfft, device=cuda)
    if name in FRAME:
        assert plan.N == FRAME[name]
    ws = wa.ws.astype(np.float64)
    fh = plan.psf_spectrum(t(f, cuda))
    xh_fwd = plan.empty_spectrum()
    y = plan.forward_image(t(x, cuda), fh, xhat_out=xh_fwd).cpu().numpy()
    y_ref = eff64.forward(x, f, g, ws)
    assert rel(y, y_ref) < TOL, name
    xh = plan.image_spectrum(t(x, cuda))
    assert rel(plan.forward_psf(t(f, cuda), xh).cpu().numpy(), y_ref) < TOL
    assert rel(xh_fwd.cpu().numpy(), xh.cpu().numpy()) < 1e-6
    gx, gf = plan.adjoint(t(r, cuda), fh, xh)
    assert rel(gx.cpu().numpy(), eff64.adjoint_image(r, f, g, ws)) < TOL
    assert rel(gf.cpu().numpy(), eff64.adjoint_psf(r, x, g, ws)) < TOL
    # fused forward from raw (x, f): same y, both spectra
    xh2, fh2 = plan.empty_spectrum(), plan.empty_spectrum()
    y2 = plan.forward_both(t(x, cuda), t(f, cuda), xhat_out=xh2, fhat_out=fh2).cpu().numpy()
    assert rel(y2, y_ref) < TOL
    assert rel(xh2.cpu().numpy(), xh.cpu().numpy()) < 1e-6
    assert rel(fh2.cpu().numpy(), fh.cpu().numpy()) < 1e-6
    # fused loss/gradient step: residual formed in-kernel, loss in FP64
    y_obs = (y_ref + r).astype(np.float32)
    loss, gx2, gf2 = plan.loss_grad(t(x, cuda), t(f, cuda), t(y_obs, cuda))
    res32 = y2.astype(np.float64) - y_obs
    assert abs(float(loss) - 0.5 * np.sum(res32 ** 2)) < 1e-5 * 0.5 * np.sum(res32 ** 2)
    assert rel(gx2.cpu().numpy(), eff64.adjoint_image(res32, f, g, ws)) < TOL
    assert rel(gf2.cpu().numpy(), eff64.adjoint_psf(res32, x, g, ws)) < TOL
    loss3, gx3, gf3 = plan.adjoint_residual(t(y2, cuda), t(y_obs, cuda), fh, xh)
    assert abs(float(loss3) - float(loss)) < 1e-5 * float(loss)
    assert rel(gx3.cpu().numpy(), gx2.cpu().numpy()) < 1e-5
    assert rel(gf3.cpu().numpy(), gf2.cpu().numpy()) < 1e-5
    # the step's two kernels on their own: residual formed by the forward,
    # adjoint and loss of that one plane
    xh4, fh4 = plan.empty_spectrum(), plan.empty_spectrum()
    r4 = plan.forward_both(t(x, cuda), t(f, cuda), xhat_out=xh4, fhat_out=fh4, subtract=t(y_obs, cuda))
    assert rel(r4.cpu().numpy(), y_ref - y_obs.astype(np.float64)) < TOL
    loss4, gx4, gf4 = plan.adjoint(r4, fh4, xh4, residual=True)
    assert abs(float(loss4) - float(loss)) < 1e-6 * float(loss)
    assert rel(gx4.cpu().numpy(), gx2.cpu().numpy()) < 1e-6
    assert rel(gf4.cpu().numpy(), gf2.cpu().numpy()) < 1e-6
    if g.mode != "full":
        gx, gf = plan.adjoint(t(r, cuda), fh, xh, adjoint="reference")
        assert rel(gx.cpu().numpy(), eff64.adjoint_image(r, f, g, ws, exact=False)) < TOL
        assert rel(gf.cpu().numpy(), eff64.adjoint_psf(r, x, g, ws, exact=False)) < TOL
    assert plan.device_errors() == 0


def test_2048_stress_workload(cuda):
    """2048x2048 image, 16x16 grid of 192x192 patches (hop 96), 41x41 motion
    PSFs, frame 256: one CTA's frame would need 240 KB of shared memory, so
    every call runs on 2-CTA clusters.  Forward against the FP64 oracle at
    full size; both adjoints through the adjoint identity."""
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(sx=(2048, 2048), csf=(16, 16), sf=(41, 41), sw=(192, 192), hop=(96, 96),
                          kind="motion", seed=21)
    plan = EffPlan(wa, g.sf, device=cuda)
    assert plan.N == 256
    xh, fh = plan.empty_spectrum(), plan.empty_spectrum()
    y = plan.forward_both(t(x, cuda), t(f, cuda), xhat_out=xh, fhat_out=fh)
    assert rel(y.cpu().numpy(), eff64.forward(x, f, g, wa.ws.astype(np.float64))) < TOL
    gx, gf = plan.adjoint(t(r, cuda), fh, xh)
    lhs = np.vdot(y.double().cpu().numpy(), r)
    assert abs(lhs - np.vdot(x, gx.double().cpu().numpy())) < 1e-5 * abs(lhs)
    assert abs(lhs - np.vdot(f, gf.double().cpu().numpy())) < 1e-5 * abs(lhs)


def test_2048_winaux_stress_workload(cuda):
    """The stress image on win2winaux's own geometry: 2088x2088 (valid output
    2048x2048), 16x16 grid of 246x246 patches (hop 123), 41x41 motion PSFs,
    extent 286: frame 512 on 8-CTA clusters.  Forward against the FP64
    oracle at full size; both adjoints through the adjoint identity."""
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(sx=(2088, 2088), csf=(16, 16), sf=(41, 41), kind="motion", seed=23)
    assert tuple(wa.sw) == (246, 246)
    plan = EffPlan(wa, g.sf, device=cuda)
    assert plan.N == 512
    xh, fh = plan.empty_spectrum(), plan.empty_spectrum()
    y = plan.forward_both(t(x, cuda), t(f, cuda), xhat_out=xh, fhat_out=fh)
    assert rel(y.cpu().numpy(), eff64.forward(x, f, g, wa.ws.astype(np.float64))) < TOL
    gx, gf = plan.adjoint(t(r, cuda), fh, xh)
    lhs = np.vdot(y.double().cpu().numpy(), r)
    assert abs(lhs - np.vdot(x, gx.double().cpu().numpy())) < 1e-5 * abs(lhs)
    assert abs(lhs - np.vdot(f, gf.double().cpu().numpy())) < 1e-5 * abs(lhs)


def test_psf_spectrum_matches_numpy_fft(cuda):
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(**CASES["cfg2_literal"])
    plan = EffPlan(wa, g.sf, device=cuda)
    fh = plan.psf_spectrum(t(f, cuda)).cpu().numpy()  # [K, N/2+1, N]: column-major half spectrum
    N = plan.N
    ref = np.fft.rfft2(eff64.pad_stack(f, (N, N)))  # [K, N, N/2+1]
    assert rel(fh, np.transpose(ref, (0, 2, 1))) < 1e-6


def test_batched_launch_matches_single(cuda):
    import torch
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(**CASES["cfg1_literal"])
    plan = EffPlan(wa, g.sf, device=cuda)
    B = 3
    xs = np.stack([synth.blob_edge_image(g.sx, seed=s) for s in range(B)])
    fs = np.stack([synth.gaussian_psfs(g.K, g.sf, seed=s + 9) for s in range(B)])
    rs = np.random.default_rng(0).standard_normal((B,) + g.sy).astype(np.float32)
    fh = plan.psf_spectrum(t(fs, cuda))
    xh = plan.empty_spectrum(B)
    y = plan.forward_image(t(xs, cuda), fh, xhat_out=xh)
    gx, gf = plan.adjoint(t(rs, cuda), fh, xh)
    for b in range(B):
        fh1 = plan.psf_spectrum(t(fs[b], cuda))
        xh1 = plan.image_spectrum(t(xs[b], cuda))
        assert rel(y[b].cpu().numpy(), plan.forward_image(t(xs[b], cuda), fh1).cpu().numpy()) < 1e-6
        gx1, gf1 = plan.adjoint(t(rs[b], cuda), fh1, xh1)
        assert rel(gx[b].cpu().numpy(), gx1.cpu().numpy()) < 1e-6
        assert rel(gf[b].cpu().numpy(), gf1.cpu().numpy()) < 1e-6
    # batched loss/gradient step (residual formed per image by the forward)
    yo = y + t(rs, cuda)
    lb, gxb, gfb = plan.loss_grad(t(xs, cuda), t(fs, cuda), yo)
    for b in range(B):
        l1, gx1, gf1 = plan.loss_grad(t(xs[b], cuda), t(fs[b], cuda), yo[b])
        assert abs(float(lb[b]) - float(l1)) < 1e-6 * float(l1)
        assert rel(gxb[b].cpu().numpy(), gx1.cpu().numpy()) < 1e-6
        assert rel(gfb[b].cpu().numpy(), gf1.cpu().numpy()) < 1e-6
        assert abs(float(l1) - 0.5 * float((rs[b].astype(np.float64) ** 2).sum())) < 1e-4 * float(l1)
    torch.cuda.synchronize()


@pytest.mark.parametrize("name", ["cfg2_literal", "cfg2_winaux"])
def test_adjoint_identity_on_gpu(cuda, name):
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(**CASES[name])
    plan = EffPlan(wa, g.sf, device=cuda)
    fh = plan.psf_spectrum(t(f, cuda))
    xh = plan.image_spectrum(t(x, cuda))
    y = plan.forward_image(t(x, cuda), fh).double().cpu().numpy()
    gx, gf = plan.adjoint(t(r, cuda), fh, xh)
    lhs = np.vdot(y, r)
    assert abs(lhs - np.vdot(x, gx.double().cpu().numpy())) < 1e-5 * abs(lhs)
    assert abs(lhs - np.vdot(f, gf.double().cpu().numpy())) < 1e-5 * abs(lhs)


def test_delta_psf_identity_on_gpu(cuda):
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(**CASES["cfg2_literal"])
    plan = EffPlan(wa, g.sf, device=cuda)
    d = np.zeros_like(f)
    d[:, 0, 0] = 1
    y = plan.forward_image(t(x, cuda), plan.psf_spectrum(t(d, cuda))).cpu().numpy()
    o = g.off
    cov = tuple(min(g.sy[k], g.sxp[k] - o[k]) for k in range(2))  # region the grid covers
    assert np.abs(y[:cov[0], :cov[1]] - x[o[0]:o[0] + cov[0], o[1]:o[1] + cov[1]]).max() < 1e-5
    # the full-convolution tail of the last patches: ~0 up to FFT rounding
    full = tuple(g.sxp[k] + g.sf[k] - 1 - o[k] for k in range(2))
    assert np.abs(y[cov[0]:full[0], :]).max() < 1e-6 and np.abs(y[:, cov[1]:full[1]]).max() < 1e-6
    # beyond the overlap-added extent nothing is written: exactly 0
    assert np.all(y[full[0]:, :] == 0) and np.all(y[:, full[1]:] == 0)


def test_repeatable_psf_adjoint(cuda):
    # the PSF adjoint uses no atomics: bitwise identical across runs
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(**CASES["cfg1_literal"])
    plan = EffPlan(wa, g.sf, device=cuda)
    xh = plan.image_spectrum(t(x, cuda))
    a = plan.adjoint(t(r, cuda), xhat=xh, want_image=False)[1]
    b = plan.adjoint(t(r, cuda), xhat=xh, want_image=False)[1]
    assert bool((a == b).all())


# ---------------------------------------------------------------------------
# projections
# ---------------------------------------------------------------------------
def test_simplex_projection(cuda):
    from vmbd_gb300.eff import project_psf
    rng = np.random.default_rng(7)
    f = rng.standard_normal((64, 25, 25)).astype(np.float32) * 0.05 + 1.0 / 625
    f[3] = -1.0  # all negative
    f[5] = 0.0
    f[6, 3, 4] = 50.0  # one dominant entry
    out = project_psf(t(f, cuda), "simplex").cpu().numpy()
    ref = eff64.simplex_project(f)
    assert np.abs(out - ref).max() < 2e-6
    assert np.allclose(out.reshape(64, -1).sum(1), 1, atol=1e-5)


def test_clip_normalize_projection(cuda):
    from vmbd_gb300.eff import project_psf
    rng = np.random.default_rng(8)
    f = rng.standard_normal((16, 31, 31)).astype(np.float32)
    f[2] = -abs(f[2])  # sums to 0 after clipping: left at 0
    out = project_psf(t(f, cuda), "clip_normalize").cpu().numpy()
    assert np.abs(out - eff64.clip_normalize(f)).max() < 1e-6


def test_basis_project(cuda):
    from vmbd_gb300.eff import basis_project
    rng = np.random.default_rng(9)
    fs = rng.standard_normal((25, 25)).astype(np.float32)
    basis = rng.standard_normal((37, 25, 25)).astype(np.float32)
    w = basis_project(t(fs, cuda), t(basis, cuda)).cpu().numpy()
    assert rel(w, eff64.basis_project(fs, basis)) < 1e-5


# ---------------------------------------------------------------------------
# autograd
# ---------------------------------------------------------------------------
def test_autograd_gradients_and_finite_differences(cuda):
    import torch
    from vmbd_gb300.autograd import eff
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(**CASES["cfg2_literal"])
    ws = wa.ws.astype(np.float64)
    y64 = eff64.forward(x, f, g, ws)
    y_obs = (y64 + 0.01 * np.random.default_rng(3).standard_normal(g.sy)).astype(np.float32)
    plan = EffPlan(wa, g.sf, device=cuda)
    xt = t(x, cuda).requires_grad_()
    ft = t(f, cuda).requires_grad_()
    yt = t(y_obs, cuda)
    y32 = eff(xt, ft, plan)
    loss = 0.5 * ((y32 - yt) ** 2).sum()
    loss.backward()
    # (1) the backward kernels: oracle adjoints of the same residual
    res32 = y32.detach().double().cpu().numpy() - y_obs
    assert rel(xt.grad.cpu().numpy(), eff64.adjoint_image(res32, f, g, ws)) < TOL
    assert rel(ft.grad.cpu().numpy(), eff64.adjoint_psf(res32, x, g, ws)) < TOL
    # (2) the whole FP32 pipeline against the FP64 one: near the optimum the
    # residual is noise-sized (sigma 0.01), so the forward's ~1e-7 rounding
    # of y is amplified in y - y_obs; bound it by that amplification
    res64 = y64 - y_obs
    amp = np.linalg.norm(res32 - res64) / np.linalg.norm(res64)
    assert amp < 1e-4
    assert rel(xt.grad.cpu().numpy(), eff64.adjoint_image(res64, f, g, ws)) < max(TOL, 100 * amp)
    assert rel(ft.grad.cpu().numpy(), eff64.adjoint_psf(res64, x, g, ws)) < max(TOL, 100 * amp)

    # (3) central finite differences, h = 1e-3, 200 random coordinates of x
    # and f, through the FP32 forward with the loss accumulated in FP64.  The
    # loss is quadratic, so the difference quotient is exact up to rounding;
    # the tolerance is the loss's rounding error divided by h: the larger of
    # its spread over repeated evaluations (atomic order) and its distance
    # from the FP64 loss (the rounding pattern itself, which a perturbed
    # input changes).
    rng = np.random.default_rng(4)
    h = 1e-3

    def loss64(xv, fv):
        with torch.no_grad():
            yv = plan.forward_image(t(xv, cuda), plan.psf_spectrum(t(fv, cuda))).double().cpu().numpy()
        return 0.5 * np.sum((yv - y_obs) ** 2)

    base = [loss64(x, f) for _ in range(8)]
    loss_fp64 = 0.5 * np.sum((y64 - y_obs) ** 2)
    sigma = max(np.std(base), abs(np.mean(base) - loss_fp64), 1e-7 * abs(base[0]) * 1e-3)
    gx = xt.grad.double().cpu().numpy()
    gf = ft.grad.double().cpu().numpy()
    fd, an = [], []
    for _ in range(100):
        i = tuple(int(rng.integers(0, s)) for s in g.sx)
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fd.append((loss64(xp, f) - loss64(xm, f)) / (2 * h))
        an.append(gx[i])
    for _ in range(100):
        i = tuple(int(rng.integers(0, s)) for s in (g.K,) + g.sf)
        fp, fm = f.copy(), f.copy()
        fp[i] += h
        fm[i] -= h
        fd.append((loss64(x, fp) - loss64(x, fm)) / (2 * h))
        an.append(gf[i])
    fd, an = np.array(fd), np.array(an)
    tol = 6 * sigma / (2 * h) + 1e-3 * np.abs(an)
    assert np.mean(np.abs(fd - an) <= tol) >= 0.95, (sigma, np.abs(fd - an).max())
    assert rel(fd, an) < 0.05


def test_reference_error_behaviour(cuda):
    from vmbd_gb300 import OlaGPU
    wa = geometry.win2winaux((96, 96), (2, 2))
    f = synth.gaussian_psfs(4, (9, 9))
    with pytest.raises(IOError):
        OlaGPU(synth.gaussian_psfs(3, (9, 9)), (96, 96), "valid", wa)
    with pytest.raises(IOError):
        OlaGPU(f, (90, 96), "valid", wa)
    with pytest.raises(NotImplementedError):
        OlaGPU(f, (96, 96), "circ", wa)
    F = OlaGPU(f, (96, 96), "full", wa)
    with pytest.raises(NotImplementedError):
        F.cnvtp(np.zeros((104, 104), np.float32))
    F = OlaGPU(f, (96, 96), "valid", wa)
    with pytest.raises(IOError):
        F.cnv(np.zeros((95, 96), np.float32))


def test_chained_call_entry_points(cuda):
    """eff_forward_ex / eff_adjoint_ex: the same results as the plain entry
    points, outputs taken as already zero when flagged, and the side-job
    buffers cleared."""
    import ctypes
    import torch
    from vmbd_gb300 import _lib
    from vmbd_gb300.eff import EffPlan, _ptr
    wa, g, x, f, r = make(**CASES["cfg1_literal"])
    plan = EffPlan(wa, g.sf, g.mode, device=cuda)
    L = _lib.load()
    st = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    xt, ft, rt = t(x, cuda), t(f, cuda), t(r, cuda)
    fh, xh = plan.psf_spectrum(ft), plan.image_spectrum(xt)
    y_img = plan.forward_image(xt, fh)
    y_psf = plan.forward_psf(ft, xh)
    for operand, u, spec, want in ((_lib.OPERAND_IMAGE, xt, fh, y_img), (_lib.OPERAND_PSF, ft, xh, y_psf)):
        for flags in (0, _lib.OUT_ZEROED):
            y = torch.zeros_like(want) if flags else torch.full_like(want, 7.0)
            side_f = torch.ones(12345, device=cuda)
            side_d = torch.ones(3, dtype=torch.float64, device=cuda)
            _lib.check(L.eff_forward_ex(plan._h, operand, _ptr(u), _ptr(spec), _ptr(y), None, None, flags,
                                        _ptr(side_f), side_f.numel(), _ptr(side_d), 3, 1, st))
            assert rel(y.cpu(), want.cpu()) < 1e-6
            assert not side_f.any() and not side_d.any()
            # residual against an observation, formed by the same kernel
            res = torch.zeros_like(want) if flags else torch.full_like(want, 7.0)
            _lib.check(L.eff_forward_ex(plan._h, operand, _ptr(u), _ptr(spec), _ptr(res), _ptr(rt), None, flags,
                                        None, 0, None, 0, 1, st))
            assert rel(res.cpu(), (want - rt).cpu()) < 1e-6
    mask = (torch.rand(plan.sy, device=cuda, generator=torch.Generator(device=cuda).manual_seed(3)) > 0.3).float()
    gx_ref, _ = plan.adjoint(rt * mask, fh, xh, want_psf=False)
    yo = 0.5 * rt
    loss_ref, _, gf_ref = plan.adjoint_residual(rt, yo, fh, xh, want_image=False)
    for flags in (0, _lib.OUT_ZEROED):
        gx = torch.zeros(plan.sx, device=cuda) if flags else torch.full(plan.sx, 3.0, device=cuda)
        _lib.check(L.eff_adjoint_ex(plan._h, _ptr(rt), None, _ptr(mask), _ptr(fh), None, _ptr(gx), None, None,
                                    _lib.ADJ_EXACT, flags, 1, st))
        assert rel(gx.cpu(), gx_ref.cpu()) < 1e-6
        loss = torch.zeros((), dtype=torch.float64, device=cuda) if flags else torch.ones((), dtype=torch.float64,
                                                                                          device=cuda)
        gf = torch.empty((plan.K,) + plan.sf, device=cuda)
        _lib.check(L.eff_adjoint_ex(plan._h, _ptr(rt), _ptr(yo), None, None, _ptr(xh), None, _ptr(gf),
                                    _ptr(loss), _lib.ADJ_EXACT, flags, 1, st))
        assert rel(gf.cpu(), gf_ref.cpu()) < 1e-6
        assert abs(float(loss) - float(loss_ref)) < 1e-6 * float(loss_ref)
    assert L.eff_forward_ex(plan._h, 5, _ptr(xt), _ptr(fh), _ptr(y_img), None, None, 0, None, 0, None, 0, 1, st) \
        == _lib.EFF_ERR_INVALID
    assert L.eff_forward_ex(plan._h, _lib.OPERAND_IMAGE, _ptr(xt), _ptr(fh), _ptr(y_img), _ptr(y_img), None, 0,
                            None, 0, None, 0, 1, st) == _lib.EFF_ERR_INVALID
    assert L.eff_adjoint_ex(plan._h, _ptr(rt), None, None, _ptr(fh), None, _ptr(gx_ref), None, None,
                            _lib.ADJ_EXACT, 8, 1, st) == _lib.EFF_ERR_INVALID
    # EFF_AFTER_FORWARD: the adjoint launched to overlap the forward it follows
    # (it waits for the forward's results on the device) gives the same output
    res = torch.zeros_like(y_img)
    _lib.check(L.eff_forward_ex(plan._h, _lib.OPERAND_IMAGE, _ptr(xt), _ptr(fh), _ptr(res), _ptr(rt), None,
                                _lib.OUT_ZEROED, None, 0, None, 0, 1, st))
    gx_pdl = torch.full(plan.sx, 3.0, device=cuda)
    _lib.check(L.eff_adjoint_ex(plan._h, _ptr(res), None, None, _ptr(fh), None, _ptr(gx_pdl), None, None,
                                _lib.ADJ_EXACT, _lib.AFTER_FORWARD, 1, st))
    gx_plain, _ = plan.adjoint(res, fh, xh, want_psf=False)
    assert rel(gx_pdl.cpu(), gx_plain.cpu()) < 1e-6


def test_cleared_outputs_at_unaligned_offsets(cuda):
    """Accumulated outputs are cleared by a small kernel (4-byte words up to
    the first 16-byte boundary, 16-byte stores, 4-byte words after the last)
    that the operator's kernel overlaps: outputs starting 4, 8 and 12 bytes
    past a boundary, in buffers full of garbage, get the results of fresh
    aligned ones, and nothing outside them is written."""
    import torch
    from vmbd_gb300.eff import EffPlan
    wa, g, x, f, r = make(**CASES["cfg1_literal"])
    plan = EffPlan(wa, g.sf, g.mode, device=cuda)
    xt, ft, rt = t(x, cuda), t(f, cuda), t(r, cuda)
    fh, xh = plan.psf_spectrum(ft), plan.image_spectrum(xt)
    yo = 0.5 * rt
    y_ref = plan.forward_image(xt, fh)
    loss_ref, gx_ref, _ = plan.adjoint_residual(rt, yo, fh, xh, want_psf=False)
    u_ref, _ = plan.deconv_xdirect(rt, fhat=fh, alpha=0.01, beta=0.01)
    ny, nx = int(np.prod(plan.sy)), int(np.prod(plan.sx))
    for off in (1, 2, 3):
        buf = torch.full((ny + 8,), 7.0, device=cuda)
        y = buf[off:off + ny].view(plan.sy)
        plan.forward_image(xt, fh, out=y)
        assert rel(y.cpu(), y_ref.cpu()) < 1e-6
        assert bool((buf[:off] == 7.0).all()) and bool((buf[off + ny:] == 7.0).all())
        gbuf = torch.full((nx + 8,), 3.0, device=cuda)
        gx = gbuf[off:off + nx].view(plan.sx)
        lbuf = torch.full((4,), 5.0, dtype=torch.float64, device=cuda)
        loss = lbuf[off]
        plan.adjoint_residual(rt, yo, fh, xh, want_psf=False, gx=gx, loss=loss)
        assert rel(gx.cpu(), gx_ref.cpu()) < 1e-6
        assert bool((gbuf[:off] == 3.0).all()) and bool((gbuf[off + nx:] == 3.0).all())
        assert abs(float(loss) - float(loss_ref)) < 1e-6 * float(loss_ref)
        assert int((lbuf == 5.0).sum()) == 3
        ubuf = torch.full((nx + 8,), 9.0, device=cuda)
        u = ubuf[off:off + nx].view(plan.sx)
        plan.deconv_xdirect(rt, fhat=fh, alpha=0.01, beta=0.01, u=u)
        assert rel(u.cpu(), u_ref.cpu()) < 1e-6
        assert bool((ubuf[:off] == 9.0).all()) and bool((ubuf[off + nx:] == 9.0).all())


@pytest.mark.parametrize("name", ["cfg1_literal", "cfg2_literal", "cfg2_winaux", "tile_odd", "tile_odd_same"])
def test_image_tile_copy_matches_lane_loads(cuda, name):
    """Kernels reading the image either copy each CTA's rows of the patch
    window into shared memory with one tensor-engine copy (x 16-byte
    aligned, image width and hop multiples of 4) or load every value
    themselves: the same values go through the same arithmetic, so the
    results are bit-identical (batched launches included)."""
    import torch
    from vmbd_gb300 import _lib
    from vmbd_gb300.eff import EffPlan
    L = _lib.load()
    spec = dict(CASES[name])
    wa, g, x, f, r = make(**spec)
    plan = EffPlan(wa, g.sf, g.mode, device=cuda)
    xs = np.stack([x, x[::-1].copy()])
    xt, ft, xbt = t(x, cuda), t(f, cuda), t(xs, cuda)
    fh = plan.psf_spectrum(ft)
    out = {}
    try:
        for on in (0, 1):
            _lib.check(L.eff_set_image_tile(on), L)
            xh = plan.empty_spectrum()
            y = plan.forward_image(xt, fh, xhat_out=xh)
            xh2, fh2 = plan.empty_spectrum(), plan.empty_spectrum()
            y2 = plan.forward_both(xt, ft, xhat_out=xh2, fhat_out=fh2)
            xs_h = plan.image_spectrum(xbt)
            out[on] = [v.cpu() for v in (y, xh, y2, xh2, xs_h)]
    finally:
        _lib.check(L.eff_set_image_tile(1), L)
    for a, b in zip(out[0], out[1]):
        # forwards overlap-add with atomics (order may differ): 1e-6; spectra exact
        if a.is_complex():
            assert torch.equal(a, b)
        else:
            assert rel(a.numpy(), b.numpy()) < 1e-6
    assert rel(out[1][0].numpy(), eff64.forward(x, f, g, wa.ws.astype(np.float64))) < TOL
    assert plan.device_errors() == 0
