"""Generate the golden EFF fixtures in this directory from the reference.

Runs the reference's own ``win2winaux``, ``OlaGPU.__init__/cnv/cnvtp/deconv``
and ``gputools`` wrappers over its ``gputools.cu`` kernels compiled for the CPU
(``oracle/ref_harness.py``; pyfft replaced by a complex64 numpy FFT), in FP32
as the reference computes, on small seeded cases, and stores inputs and
outputs as ``ref_<case>.npz``.

Entries the reference leaves undefined are stored as NaN: where the patch grid
covers less than the image, ``crop_gpu2cpu`` reads beyond the overlap-added
array (no source bounds check in crop_Kernel, gputools.cu:254-263).

Needs the reference checkout; run ``python tests/golden/make_golden.py [case ...]``
(all cases when none is named).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_harness as rh  # noqa: E402
from vmbd_gb300 import synth  # noqa: E402

# name: (sx, csf, sf, mode, winaux_sx (None: the image size), psf kind, seed)
# winaux_sx: the window stack is that of win2winaux on a smaller image whose
# patch size is the literal one (hop*(csf-1) + sw), used on the full image.
CASES = {
    "valid_mixed_parity": ((60, 52), (3, 2), (7, 5), "valid", None, "gauss", 11),
    "literal_uncovered": ((64, 64), (2, 2), (9, 9), "valid", (36, 36), "motion", 12),
    "same_even_psf": ((50, 70), (2, 3), (6, 8), "same", None, "gauss", 13),
    "grid4x4_sf15": ((96, 96), (4, 4), (15, 15), "valid", None, "gauss", 14),
    "wide_nonsquare": ((40, 120), (2, 5), (5, 11), "valid", None, "motion", 15),
}
# The two literal workload geometries: 256x256 with a 4x4 grid of 64x64
# patches and 15x15 Gaussian PSFs, and 512x512 with an 8x8 grid of 96x96
# patches and 31x31 motion PSFs (both frame 128).  Stored compact: the image
# and PSFs are stored (the generators' rounding differs between machines),
# the residual is regenerated from its seed (numpy's generator is the same
# everywhere) and pinned by a checksum, the window stack is the host
# geometry's.
LARGE_CASES = {
    "cfg1_literal": ((256, 256), (4, 4), (15, 15), "valid", (160, 160), "gauss", 31),
    "cfg2_literal": ((512, 512), (8, 8), (31, 31), "valid", (432, 432), "motion", 32),
}


def make_case(name, sx, csf, sf, mode, wa_sx, kind, seed, gputools, imagetools, olaGPU, compact=False):
    sx = np.array(sx)
    sf = np.array(sf)
    K = int(np.prod(csf))
    wa = imagetools.win2winaux(np.array(wa_sx if wa_sx else sx), csf, 0.5)
    wa.sx = sx  # literal geometry: the window stack of a smaller grid on this image
    x = synth.blob_edge_image(tuple(sx), seed=seed)
    gen = synth.gaussian_psfs if kind == "gauss" else synth.motion_psfs
    f = gen(K, tuple(sf), seed=seed + 100)

    F = olaGPU.OlaGPU(f, sx, mode, wa)
    y = F.cnv(x)
    X = olaGPU.OlaGPU(rh.cua.to_gpu(x), sf, mode, wa)
    yX = None if compact else X.cnv(f)
    r = np.random.default_rng(seed + 200).standard_normal(y.shape).astype(np.float32)
    gx = F.cnvtp(rh.cua.to_gpu(r)).get()
    gf = X.cnvtp(rh.cua.to_gpu(r)).get()

    sw = np.array(wa.sw, dtype=int)
    hop = np.array(wa.nhop, dtype=int)
    sxp = hop * np.array(csf) + sw - hop
    off = {"valid": sf - 1, "same": sf // 2, "full": 0 * sf}[mode]
    yfull = sxp + sf - 1
    ii, jj = np.meshgrid(np.arange(y.shape[0]), np.arange(y.shape[1]), indexing="ij")
    undefined_y = (ii + off[0] >= yfull[0]) | (jj + off[1] >= yfull[1])
    ii, jj = np.meshgrid(np.arange(sx[0]), np.arange(sx[1]), indexing="ij")
    undefined_x = (ii >= sxp[0]) | (jj >= sxp[1])
    for a, m in ((y, undefined_y), (yX, undefined_y), (gx, undefined_x)):
        if a is not None:
            a[m] = np.nan
    out = dict(sx=sx, sf=sf, csf=np.array(csf), sw=sw, hop=hop, mode=np.array(mode),
               sfft=np.array(F.sfft_gpu), y=y.astype(np.float32), gx=gx.astype(np.float32),
               gf=gf.astype(np.float32))
    if compact:
        # the residual is regenerated from the seed; its checksum pins it
        out.update(x=x, f=f, seed=np.array(seed),
                   r_sum=np.array([np.sum(r, dtype=np.float64), np.sum(np.square(r, dtype=np.float64))]))
    else:
        out.update(x=x, f=f, r=r, ws=np.asarray(wa.ws_gpu, np.float32), yX=yX.astype(np.float32))
    path = os.path.join(HERE, f"ref_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: sx={tuple(sx)} csf={csf} sf={tuple(sf)} sw={tuple(sw)} hop={tuple(hop)} "
          f"sfft={F.sfft_gpu} mode={mode} -> {os.path.basename(path)}")


# Fourier-division deconvolution, OlaGPU.deconv(mode='xdirect') of an F object
# (image estimate) and of an X object (PSF estimate):
# name: (sx, csf, sf, mode, psf kind, seed, alpha, beta)
DECONV_CASES = {
    "deconv_valid": ((96, 96), (2, 2), (9, 9), "valid", "gauss", 21, 0.0, 0.01),
    "deconv_same_laplacian": ((80, 112), (2, 3), (7, 7), "same", "motion", 22, 0.05, 1e-3),
    "deconv_grid4x4": ((96, 96), (4, 4), (15, 15), "valid", "gauss", 23, 0.01, 0.01),
}


def make_deconv_case(name, sx, csf, sf, mode, kind, seed, alpha, beta, imagetools, olaGPU):
    sx = np.array(sx)
    sf = np.array(sf)
    K = int(np.prod(csf))
    wa = imagetools.win2winaux(sx, csf, 0.5)
    x = synth.blob_edge_image(tuple(sx), seed=seed)
    gen = synth.gaussian_psfs if kind == "gauss" else synth.motion_psfs
    f = gen(K, tuple(sf), seed=seed + 100)
    F = olaGPU.OlaGPU(f, sx, mode, wa)
    y = np.asarray(F.cnv(x), np.float32)
    y = (y + 0.01 * np.random.default_rng(seed + 200).standard_normal(y.shape)).astype(np.float32)
    X = olaGPU.OlaGPU(rh.cua.to_gpu(x), sf, mode, wa)
    # edgetapering=0: the taper in 'xdirect' acts on a copy the chop never
    # reads (olaGPU.py:566-575), so the result is the same without it
    u = np.asarray(F.deconv(y, mode="xdirect", alpha=alpha, beta=beta, edgetapering=0), np.float32)
    fz = np.asarray(X.deconv(y, mode="xdirect", alpha=alpha, beta=beta, edgetapering=0), np.float32)
    assert np.isfinite(u).all() and np.isfinite(fz).all()
    out = dict(sx=sx, sf=sf, csf=np.array(csf), sw=np.array(wa.sw, dtype=int),
               hop=np.array(wa.nhop, dtype=int), mode=np.array(mode), sfft=np.array(F.sfft_gpu),
               alpha=np.array(alpha), beta=np.array(beta), x=x, f=f, y=y,
               ws=np.asarray(wa.ws_gpu, np.float32), u=u, fz=fz)
    path = os.path.join(HERE, f"ref_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: sx={tuple(sx)} csf={csf} sf={tuple(sf)} sw={tuple(wa.sw)} sfft={F.sfft_gpu} "
          f"mode={mode} alpha={alpha} beta={beta} -> {os.path.basename(path)}")


def main():
    gputools, imagetools, olaGPU = rh.load()
    only = set(sys.argv[1:])
    for name, spec in CASES.items():
        if not only or name in only:
            make_case(name, *spec, gputools, imagetools, olaGPU)
    for name, spec in LARGE_CASES.items():
        if not only or name in only:
            make_case(name, *spec, gputools, imagetools, olaGPU, compact=True)
    for name, spec in DECONV_CASES.items():
        if not only or name in only:
            make_deconv_case(name, *spec, imagetools, olaGPU)


if __name__ == "__main__":
    main()
