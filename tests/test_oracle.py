"""CPU: the FP64 oracle against the reference's golden vectors and against
its own known-answer properties; the product's host-side geometry against
the oracle."""
import os
import sys

import numpy as np
import pytest

from oracle import eff64
from vmbd_gb300 import geometry, synth

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import fixtures  # noqa: E402

# operator fixtures (cnv / cnvtp) and Fourier-division deconvolution fixtures
GOLDEN = fixtures.operator_paths()
DECONV_GOLDEN = fixtures.deconv_paths()


def load_case(path):
    d = fixtures.load(path)
    d["geom"] = eff64.Geometry(tuple(d["sx"]), tuple(d["sf"]), tuple(d["csf"]), tuple(d["sw"]),
                               tuple(d["hop"]), d["mode"])
    return d


def rel(a, b, mask=None):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_golden_present():
    assert len(GOLDEN) >= 5
    names = {os.path.basename(p) for p in GOLDEN}
    # the literal workload geometries: 256^2 / 4x4 x 64^2 / 15^2 and 512^2 / 8x8 x 96^2 / 31^2
    assert {"ref_cfg1_literal.npz", "ref_cfg2_literal.npz"} <= names


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p))
def test_oracle_matches_reference_forward(path):
    c = load_case(path)
    g = c["geom"]
    ws = c["ws"].astype(np.float64)
    y = eff64.forward(c["x"], c["f"], g, ws)
    m = np.isfinite(c["y"])
    # reference computes in FP32: tolerance is FP32 rounding of the pipeline
    assert rel(y, c["y"], m) < 2e-6
    if "yX" in c:  # X.cnv of the same operator (small cases)
        assert rel(y, c["yX"], m) < 2e-6
    # the entries the reference leaves undefined are 0 here
    assert np.all(y[~m] == 0)


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p))
def test_oracle_matches_reference_adjoints(path):
    c = load_case(path)
    g = c["geom"]
    ws = c["ws"].astype(np.float64)
    gx = eff64.adjoint_image(c["r"], c["f"], g, ws, exact=False)
    gf = eff64.adjoint_psf(c["r"], c["x"], g, ws, exact=False)
    m = np.isfinite(c["gx"])
    assert rel(gx, c["gx"], m) < 2e-6
    assert rel(gf, c["gf"]) < 2e-6


@pytest.mark.parametrize("path", DECONV_GOLDEN, ids=lambda p: os.path.basename(p))
def test_oracle_matches_reference_xdirect(path):
    """OlaGPU.deconv(mode='xdirect') of an F object (image estimate) and of
    an X object (PSF estimate), the reference run on its own kernels; the
    reference frame (``sfft``) is the one the division happens in."""
    z = np.load(path)
    c = {k: z[k] for k in z.files}
    g = eff64.Geometry(tuple(c["sx"]), tuple(c["sf"]), tuple(c["csf"]), tuple(c["sw"]), tuple(c["hop"]),
                       str(c["mode"]), tuple(c["sfft"]))
    ws = c["ws"].astype(np.float64)
    alpha, beta = float(c["alpha"]), float(c["beta"])
    u = eff64.deconv_xdirect(c["y"], eff64.psf_spectrum(c["f"], g), g, ws, "image", alpha, beta)
    fz = eff64.deconv_xdirect(c["y"], eff64.image_spectrum(c["x"], g, ws), g, ws, "psf", alpha, beta)
    assert rel(u, c["u"]) < 2e-6
    assert rel(fz, c["fz"]) < 1e-5


def test_deconv_golden_present():
    assert len(DECONV_GOLDEN) >= 3


def test_xdirect_with_delta_psfs_returns_the_image():
    """Known answer: PSFs that are deltas at the origin have spectrum 1, so
    the division is a scaling by 1/(1 + beta) and the image estimate at pixel
    i is the overlap-add of ws_k[i - m*hop] * y[i - (sf-1)] over the patches
    whose chop (frame rows [sf-1, sw)) reaches i.  Where every covering patch
    reaches it, that sum is y[i - (sf-1)] = x[i] (partition of unity)."""
    wa = geometry.win2winaux((64, 64), (2, 2), 0.5)
    sf = (5, 5)
    g = eff64.Geometry(wa.sx, sf, wa.csf, wa.sw, wa.nhop, "valid")
    ws = wa.ws.astype(np.float64)
    x = synth.blob_edge_image(wa.sx, seed=3)
    f = np.zeros((g.K,) + sf)
    f[:, 0, 0] = 1.0
    y = eff64.forward(x, f, g, ws)
    beta = 1e-3
    u = eff64.deconv_xdirect(y, eff64.psf_spectrum(f, g), g, ws, "image", 0.0, beta)
    ok = []
    for d in range(2):
        i = np.arange(wa.sx[d])
        good = np.ones(wa.sx[d], bool)
        for m in range(wa.csf[d]):
            r = i - m * wa.nhop[d]
            covered = (r >= 0) & (r < wa.sw[d])
            good &= ~covered | (r >= sf[d] - 1)
        ok.append(good)
    mask = ok[0][:, None] & ok[1][None, :]
    assert mask.sum() > 0.5 * mask.size
    # the window stack is float32: its partition of unity holds to ~1e-7
    assert np.abs(u[mask] - x[mask] / (1 + beta)).max() < 1e-6


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p))
def test_windows_match_reference(path):
    c = load_case(path)
    wa = geometry.Winaux(tuple(c["sx"]), tuple(c["csf"]), tuple(c["sw"]), tuple(c["hop"]))
    assert np.abs(wa.ws - c["ws"]).max() < 1e-6
    wo = eff64.win2winaux(tuple(c["sx"]), tuple(c["csf"]), 0.5, tuple(c["sw"]), tuple(c["hop"]))
    assert np.abs(wo.ws - c["ws"]).max() < 1e-6
    assert np.abs(wa.ws - wo.ws).max() < 1e-6


@pytest.mark.parametrize("sx,csf", [((60, 52), (3, 2)), ((512, 512), (8, 8)), ((404, 532), (6, 8)),
                                    ((1054, 1054), (12, 12)), ((270, 270), (4, 4))])
def test_patch_geometry_matches_oracle(sx, csf):
    assert geometry.patch_geometry(sx, csf) == eff64.win2winaux_geometry(sx, csf)


def test_mixed_parity_fallback():
    # 384x512 + 20 with a 6x8 grid never reaches an integral sw*0.5 in both
    # dims: the reference falls back to the first guess.
    assert geometry.patch_geometry((404, 532), (6, 8)) == ((116, 119), (58, 60))


def small_geom(mode="valid", sx=(70, 58), csf=(3, 2), sf=(9, 7)):
    wa = eff64.win2winaux(sx, csf, 0.5)
    return eff64.geometry_from_winaux(wa, sf, mode), wa.ws


@pytest.mark.parametrize("mode", ["valid", "same", "full"])
def test_direct_summation_matches_fft(mode):
    g, ws = small_geom(mode)
    rng = np.random.default_rng(1)
    x = rng.random(g.sx)
    f = rng.random((g.K,) + g.sf)
    assert rel(eff64.forward_direct(x, f, g, ws), eff64.forward(x, f, g, ws)) < 1e-13


@pytest.mark.parametrize("mode", ["valid", "same", "full"])
def test_exact_adjoint_identity(mode):
    g, ws = small_geom(mode)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(g.sx)
    f = rng.standard_normal((g.K,) + g.sf)
    r = rng.standard_normal(g.sy)
    y = eff64.forward(x, f, g, ws)
    lhs = np.vdot(y, r)
    assert abs(lhs - np.vdot(x, eff64.adjoint_image(r, f, g, ws))) < 1e-12 * abs(lhs) * 1e3
    assert abs(lhs - np.vdot(f, eff64.adjoint_psf(r, x, g, ws))) < 1e-12 * abs(lhs) * 1e3


def test_reference_adjoint_is_not_exact():
    g, ws = small_geom("valid")
    rng = np.random.default_rng(3)
    x, f, r = rng.random(g.sx), rng.random((g.K,) + g.sf), rng.random(g.sy)
    ex = eff64.adjoint_image(r, f, g, ws, exact=True)
    rf = eff64.adjoint_image(r, f, g, ws, exact=False)
    assert 1e-4 < rel(rf, ex) < 0.2


def test_delta_psf_identity():
    g, ws = small_geom("valid")
    x = np.random.default_rng(4).random(g.sx)
    f = np.zeros((g.K,) + g.sf)
    f[:, 0, 0] = 1
    y = eff64.forward(x, f, g, ws)
    o = g.off
    assert np.abs(y - x[o[0]:o[0] + g.sy[0], o[1]:o[1] + g.sy[1]]).max() < 1e-12


def test_partition_of_unity():
    wa = eff64.win2winaux((70, 58), (3, 2), 0.5)
    tot = eff64.ola(wa.ws, wa.csf, wa.sw, wa.nhop)
    assert np.abs(tot - 1).max() < 1e-12


def test_simplex_projection_properties():
    rng = np.random.default_rng(5)
    f = rng.standard_normal((16, 9, 9))
    p = eff64.simplex_project(f)
    assert np.all(p >= 0)
    assert np.allclose(p.reshape(16, -1).sum(1), 1)
    # optimality: p is closer to f than random feasible points
    for _ in range(20):
        q = rng.random((16, 81))
        q /= q.sum(1, keepdims=True)
        assert np.all(((p.reshape(16, -1) - f.reshape(16, -1)) ** 2).sum(1) <=
                      ((q - f.reshape(16, -1)) ** 2).sum(1) + 1e-12)
    # idempotent
    assert np.allclose(eff64.simplex_project(p), p)


def test_clip_normalize():
    f = np.array([[[-1.0, 1.0], [2.0, 1.0]], [[0, 0], [0, 1e-7]]])
    p = eff64.clip_normalize(f)
    assert np.allclose(p[0], [[0, 0.25], [0.5, 0.25]])
    assert np.allclose(p[1], [[0, 0], [0, 1e-7]])  # sum below 1e-6: left alone


def test_synthetic_generators():
    img = synth.blob_edge_image((64, 80), seed=3)
    assert img.shape == (64, 80) and img.dtype == np.float32
    assert img.min() == 0 and abs(img.max() - 1) < 1e-6
    for gen in (synth.gaussian_psfs, synth.motion_psfs):
        f = gen(5, (15, 15), seed=1)
        assert f.shape == (5, 15, 15) and np.all(f >= 0)
        assert np.allclose(f.reshape(5, -1).sum(1), 1, atol=1e-5)
    assert np.array_equal(synth.blob_edge_image((32, 32), 7), synth.blob_edge_image((32, 32), 7))
    d = synth.drifting_motion_psfs(4, 3, (25, 25), seed=2)
    assert d.shape == (4, 3, 25, 25)


def test_fp64_finite_differences():
    """Central differences (h = 1e-3, 200 coordinates) of 0.5||EFF(x,f)-y||^2
    in FP64 against the exact adjoints."""
    g, ws = small_geom("valid")
    rng = np.random.default_rng(6)
    x = rng.random(g.sx)
    f = rng.random((g.K,) + g.sf)
    y = rng.random(g.sy)
    res = eff64.forward(x, f, g, ws) - y
    gx = eff64.adjoint_image(res, f, g, ws)
    gf = eff64.adjoint_psf(res, x, g, ws)

    def L(xv, fv):
        return 0.5 * np.sum((eff64.forward(xv, fv, g, ws) - y) ** 2)

    h = 1e-3
    fd, an = [], []
    for _ in range(100):
        i = tuple(int(rng.integers(0, s)) for s in g.sx)
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fd.append((L(xp, f) - L(xm, f)) / (2 * h))
        an.append(gx[i])
    for _ in range(100):
        i = tuple(int(rng.integers(0, s)) for s in (g.K,) + g.sf)
        fp, fm = f.copy(), f.copy()
        fp[i] += h
        fm[i] -= h
        fd.append((L(x, fp) - L(x, fm)) / (2 * h))
        an.append(gf[i])
    assert rel(np.array(fd), np.array(an)) < 1e-8
