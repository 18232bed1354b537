"""FP64 NumPy restatement of VMBD's efficient-filter-flow (EFF) operator.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: the CUDA path in
``vmbd_gb300`` is checked against it, and ``bench.py`` times it as the CPU
baseline.  Nothing in the product imports it.

Every function restates one piece of the reference (Python 2 + PyCUDA + pyfft,
which cannot run here) and cites the file:line it follows.  Arithmetic is
FP64; the reference computes in FP32.

Parity pinning: the index conventions of chop / pad / crop / overlap-add are
pinned against the reference's own CUDA kernels (``gputools.cu``) compiled for
the CPU into ``oracle/_ref`` (see ``oracle/ref_harness.py``) through the golden
fixtures in ``tests/golden``.  The FFT of the reference comes from pyfft 0.3.5,
a third-party package that is absent; ``numpy.fft`` (FP64) stands in for it,
so the FFT boundary itself is unpinned and is checked instead by a direct
spatial-domain summation (``forward_direct``) and the adjoint identity.

Notation (all C-order): ``K = csf0*csf1`` patches, patch ``k = m*csf1 + n``
with origin ``(m*hop0, n*hop1)``; ``E = sw + sf - 1`` is the extent of one
patch's full linear convolution; ``N`` (``sfft``) the FFT frame, ``N >= E``.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np
import scipy.fft
from scipy import signal

# FFT backend: numpy (one thread) by default; set_fft_workers(n) switches to
# scipy.fft over n threads (used when the oracle is timed as the CPU baseline).
_WORKERS = None


def set_fft_workers(n):
    global _WORKERS
    _WORKERS = n


def _rfft2(a):
    if _WORKERS:
        return scipy.fft.rfft2(a, workers=_WORKERS)
    return np.fft.rfft2(a)


def _irfft2(a, s):
    if _WORKERS:
        return scipy.fft.irfft2(a, s=s, workers=_WORKERS)
    return np.fft.irfft2(a, s=s)

# --------------------------------------------------------------------------
# Windows and geometry
# --------------------------------------------------------------------------


def window(sw, name: str = "barthann") -> np.ndarray:
    """2-D window of shape ``sw``: imagetools.py:314-344.

    Each 1-D factor is scipy's periodic window, symmetrised as
    ``(w + w[::-1]) / 2`` and shifted so its minimum is 0; the outer product
    is scaled to max 1 and floored at 1e-16.
    """
    def one(n):
        w = signal.get_window(name, int(n))
        w = (w + w[::-1]) / 2
        return w - w.min()

    w = np.outer(one(sw[0]), one(sw[1]))
    w = w / w.max()
    return np.maximum(w, 1e-16)


def pow2_frame(e) -> tuple:
    """``2**ceil(log2(e))`` per dim: olaGPU.py:139-141."""
    return tuple(int(2 ** math.ceil(math.log2(int(v)))) for v in e)


@dataclasses.dataclass
class Winaux:
    """Result of ``win2winaux``: imagetools.py:398-454."""
    sx: tuple
    csf: tuple
    sw: tuple
    nhop: tuple
    ws: np.ndarray  # [K, sw0, sw1] partition-of-unity window stack

    @property
    def sxp(self) -> tuple:
        """Extent covered by the patch grid, ``nhop*csf + sw - nhop``
        (gputools.py:371-372)."""
        return tuple(self.nhop[d] * self.csf[d] + self.sw[d] - self.nhop[d] for d in range(2))


def win2winaux_geometry(sx, csf, overlap: float = 0.5):
    """Patch size / hop from image size: imagetools.py:422-436.

    ``sw = ceil(sx / (csf*(1-ov) + ov))``, then both dims are incremented
    together until ``sw*ov`` is integral in every dim; if that overshoots
    ``2*sw`` the original ``sw`` is kept.  ``nhop = sw - floor(sw*ov)``.
    """
    sx = np.asarray(sx, dtype=np.float64)
    csf_a = np.asarray(csf, dtype=np.float64)
    factor = csf_a * (1 - overlap) + overlap
    sw = np.ceil(sx / factor)
    swold = sw
    while np.any(np.floor(sw * overlap) != sw * overlap):
        sw = sw + 1
        if np.any(sw > 2 * swold):
            sw = swold
            break
    nhop = sw - np.floor(sw * overlap)
    return tuple(int(v) for v in sw), tuple(int(v) for v in nhop)


def win2winaux(sx, csf, overlap: float = 0.5, sw=None, nhop=None) -> Winaux:
    """Window stack ``ws = w / chop(ola(w))``: imagetools.py:437-454.

    ``sw``/``nhop`` may be given explicitly (the patch sizes a config states);
    by default they come from ``win2winaux_geometry``.  The window is always
    Bartlett-Hann, as in the reference (its ``windowfun`` argument is unused,
    imagetools.py:438).
    """
    if sw is None:
        sw, nhop = win2winaux_geometry(sx, csf, overlap)
    sw = tuple(int(v) for v in sw)
    nhop = tuple(int(v) for v in nhop)
    csf = tuple(int(v) for v in csf)
    K = csf[0] * csf[1]
    w = window(sw)
    nom = np.tile(w, (K, 1, 1))
    w_ola = ola(nom, csf, sw, nhop)
    denom = chop_pad(w_ola, csf, sw, nhop, sw)
    return Winaux(tuple(int(v) for v in sx), csf, sw, nhop, nom / denom)


# --------------------------------------------------------------------------
# Chop / pad / crop / overlap-add (the reference's index conventions)
# --------------------------------------------------------------------------


def pad_to(x: np.ndarray, sz, offset=(0, 0)) -> np.ndarray:
    """Zero-pad (or crop) ``x`` into an ``sz`` array at ``offset``:
    zeroPadKernel gputools.cu:154-166 via pad_cpu2gpu gputools.py:1099-1137."""
    out = np.zeros(tuple(int(v) for v in sz), dtype=np.float64)
    s, t = int(offset[0]), int(offset[1])
    m = min(x.shape[0], out.shape[0] - s)
    n = min(x.shape[1], out.shape[1] - t)
    if m > 0 and n > 0:
        out[s:s + m, t:t + n] = x[:m, :n]
    return out


def chop_pad(x: np.ndarray, csf, sw, nhop, sz, offset=(0, 0)) -> np.ndarray:
    """Overlapping patches of ``x`` placed in zeroed ``sz`` frames at
    ``offset``: chop_pad_Kernel gputools.cu:60-79 via chop_pad_GPU
    gputools.py:364-401.

    ``x`` is first padded/cropped to ``sxp = nhop*csf + sw - nhop`` at the
    origin (``pad_cpu2gpu``).  Patch ``k=(m,n)``: ``out[k, r+o0, c+o1] =
    xp[m*hop0 + r, n*hop1 + c]`` for ``r < sw0, c < sw1`` inside the frame.
    """
    csf = tuple(int(v) for v in csf)
    sw = tuple(int(v) for v in sw)
    nhop = tuple(int(v) for v in nhop)
    sz = tuple(int(v) for v in sz)
    sxp = tuple(nhop[d] * csf[d] + sw[d] - nhop[d] for d in range(2))
    xp = pad_to(np.asarray(x, dtype=np.float64), sxp)
    o0, o1 = int(offset[0]), int(offset[1])
    r_end = min(sw[0], sz[0] - o0)
    c_end = min(sw[1], sz[1] - o1)
    out = np.zeros((csf[0] * csf[1],) + sz, dtype=np.float64)
    for m in range(csf[0]):
        for n in range(csf[1]):
            k = m * csf[1] + n
            out[k, o0:o0 + r_end, o1:o1 + c_end] = \
                xp[m * nhop[0]:m * nhop[0] + r_end, n * nhop[1]:n * nhop[1] + c_end]
    return out


def pad_stack(x: np.ndarray, sz, offset=(0, 0)) -> np.ndarray:
    """Each slice of ``x[K, xm, xn]`` into a zeroed ``sz`` frame at
    ``offset``: pad_stack_Kernel gputools.cu:184-201 via pad_stack_GPU
    gputools.py:1140-1181."""
    sz = tuple(int(v) for v in sz)
    o0, o1 = int(offset[0]), int(offset[1])
    out = np.zeros((x.shape[0],) + sz, dtype=np.float64)
    m = min(x.shape[1], sz[0] - o0)
    n = min(x.shape[2], sz[1] - o1)
    out[:, o0:o0 + m, o1:o1 + n] = x[:, :m, :n]
    return out


def crop_stack(x: np.ndarray, sz, offset=(0, 0)) -> np.ndarray:
    """``out[k, r, c] = x[k, r+o0, c+o1]``: crop_stack_Kernel
    gputools.cu:225-236 via crop_stack_GPU gputools.py:599-640 (real part
    for complex input, gputools.py:620-621)."""
    o0, o1 = int(offset[0]), int(offset[1])
    return np.real(x[:, o0:o0 + int(sz[0]), o1:o1 + int(sz[1])]).copy()


def crop(x: np.ndarray, sz, offset=(0, 0)) -> np.ndarray:
    """``out[i, j] = x[i+s, j+t]``: crop_Kernel gputools.cu:254-263 via
    crop_gpu2cpu gputools.py:546-569.

    Output entries with no source pixel are left unwritten by the reference
    (``cua.empty``); here they are 0."""
    out = np.zeros(tuple(int(v) for v in sz), dtype=np.float64)
    s, t = int(offset[0]), int(offset[1])
    m = max(0, min(out.shape[0], x.shape[0] - s))
    n = max(0, min(out.shape[1], x.shape[1] - t))
    out[:m, :n] = np.real(x[s:s + m, t:t + n])
    return out


def ola(xs: np.ndarray, csf, ext, nhop, offset=(0, 0)) -> np.ndarray:
    """Overlap-add of a patch stack: ola_Kernel_test gputools.cu:296-314 via
    ola_GPU_test gputools.py:1068-1096.

    The output has size ``nhop*csf + ext - nhop``; pixel ``i`` sums
    ``xs[k=(m,n)][o0 + i - m*hop0, o1 + j - n*hop1]`` over the patches with
    ``0 <= i - m*hop0 < ext0`` (and likewise in the other dim).  The kernel
    writes this as a gather; the scatter below visits the same terms.
    ``ext`` must not exceed the slice size (the reference's ``F.cnvtp``
    passes a larger one, olaGPU.py:307, and reads out of bounds; callers here
    pass the in-bounds extent).
    """
    csf = tuple(int(v) for v in csf)
    ext = tuple(int(v) for v in ext)
    nhop = tuple(int(v) for v in nhop)
    o0, o1 = int(offset[0]), int(offset[1])
    if o0 + ext[0] > xs.shape[1] or o1 + ext[1] > xs.shape[2]:
        raise ValueError("ola extent exceeds the slice size")
    out = np.zeros(tuple(nhop[d] * csf[d] + ext[d] - nhop[d] for d in range(2)), dtype=np.float64)
    for m in range(csf[0]):
        for n in range(csf[1]):
            k = m * csf[1] + n
            out[m * nhop[0]:m * nhop[0] + ext[0], n * nhop[1]:n * nhop[1] + ext[1]] += \
                np.real(xs[k, o0:o0 + ext[0], o1:o1 + ext[1]])
    return out


# --------------------------------------------------------------------------
# The operator
# --------------------------------------------------------------------------

MODES = ("valid", "same", "full")


@dataclasses.dataclass
class Geometry:
    """Everything the operator needs besides the data (olaGPU.py:95-168)."""
    sx: tuple      # image size
    sf: tuple      # PSF size
    csf: tuple     # patch grid
    sw: tuple      # patch size
    hop: tuple     # patch hop
    mode: str = "valid"
    sfft: tuple = None  # FFT frame; default pow2(sw + sf - 1)

    def __post_init__(self):
        for f in ("sx", "sf", "csf", "sw", "hop"):
            setattr(self, f, tuple(int(v) for v in getattr(self, f)))
        if self.mode not in MODES:
            raise NotImplementedError("Not a valid mode!")
        if self.sfft is None:
            self.sfft = pow2_frame(self.ext)
        self.sfft = tuple(int(v) for v in self.sfft)

    @property
    def K(self) -> int:
        return self.csf[0] * self.csf[1]

    @property
    def ext(self) -> tuple:
        return tuple(self.sw[d] + self.sf[d] - 1 for d in range(2))

    @property
    def sxp(self) -> tuple:
        return tuple(self.hop[d] * self.csf[d] + self.sw[d] - self.hop[d] for d in range(2))

    @property
    def sy(self) -> tuple:
        """olaGPU.py:127-136."""
        if self.mode == "valid":
            return tuple(self.sx[d] - self.sf[d] + 1 for d in range(2))
        if self.mode == "same":
            return self.sx
        return tuple(self.sx[d] + self.sf[d] - 1 for d in range(2))

    @property
    def off(self) -> tuple:
        """Crop offset of the output inside the overlap-added full
        convolution: olaGPU.py:239-244."""
        if self.mode == "valid":
            return tuple(v - 1 for v in self.sf)
        if self.mode == "same":
            return tuple(v // 2 for v in self.sf)
        return (0, 0)


def geometry_from_winaux(wa: Winaux, sf, mode="valid", sfft=None) -> Geometry:
    return Geometry(wa.sx, sf, wa.csf, wa.sw, wa.nhop, mode, sfft)


def windowed_patches(x, g: Geometry, ws, sz) -> np.ndarray:
    """``ws_k * chop_k(x)`` in ``sz`` frames: chop_mod_pad_Kernel
    gputools.cu:16-35 (X object, olaGPU.py:147-151) and the equivalent
    chop_pad + pad_stack(ws) + multiply of ``cnv`` (olaGPU.py:210-217)."""
    return chop_pad(x, g.csf, g.sw, g.hop, sz) * pad_stack(ws, sz)


def forward(x, f, g: Geometry, ws) -> np.ndarray:
    """``y = F x = X f``: OlaGPU.cnv olaGPU.py:170-257.

    Per patch: FFT of the windowed patch times the FFT of the zero-padded
    PSF, inverse FFT (the reference forms it as conj(FFT(conj))/N,
    olaGPU.py:225-231), overlap-add with extent ``sw + sf - 1``
    (olaGPU.py:234-236), crop by mode (olaGPU.py:239-244).
    """
    N = g.sfft
    u = windowed_patches(x, g, ws, N)
    Fh = _rfft2(pad_stack(np.asarray(f, np.float64), N))
    ys = _irfft2(_rfft2(u) * Fh, s=N)
    yfull = ola(ys, g.csf, g.ext, g.hop)
    return crop(yfull, g.sy, g.off)


def forward_direct(x, f, g: Geometry, ws) -> np.ndarray:
    """Same operator by direct spatial summation (no FFT): an independent
    second oracle for ``forward``."""
    u = chop_pad(x, g.csf, g.sw, g.hop, g.sw) * ws
    full = np.zeros(tuple(g.sxp[d] + g.sf[d] - 1 for d in range(2)))
    for m in range(g.csf[0]):
        for n in range(g.csf[1]):
            k = m * g.csf[1] + n
            c = signal.convolve2d(u[k], np.asarray(f[k], np.float64), mode="full")
            full[m * g.hop[0]:m * g.hop[0] + g.ext[0], n * g.hop[1]:n * g.hop[1] + g.ext[1]] += c
    return crop(full, g.sy, g.off)


def residual_frames(y, g: Geometry, exact: bool = True) -> np.ndarray:
    """Per-patch frames of the output-side image for the adjoints.

    Reference (``exact=False``): chop_pad of ``y`` with frame offset ``off``
    and extent ``sw`` (olaGPU.py:276-286).  Exact: the full extent
    ``sw + sf - 1`` of ``y`` embedded at ``off`` in the full-convolution
    grid, i.e. ``frame[s, t] = y[m*hop0 + s - off0, n*hop1 + t - off1]`` for
    ``0 <= s < E0`` (zero outside ``y``).  The reference drops the strip
    ``s < off`` and so is not the exact transpose of ``forward``.
    """
    N = g.sfft
    if not exact:
        return chop_pad(y, g.csf, g.sw, g.hop, N, g.off)
    full_sz = tuple(g.sxp[d] + g.sf[d] - 1 for d in range(2))
    yfull = pad_to(np.asarray(y, np.float64), full_sz, g.off)
    out = np.zeros((g.K,) + tuple(N), dtype=np.float64)
    E = g.ext
    for m in range(g.csf[0]):
        for n in range(g.csf[1]):
            k = m * g.csf[1] + n
            out[k, :E[0], :E[1]] = yfull[m * g.hop[0]:m * g.hop[0] + E[0],
                                         n * g.hop[1]:n * g.hop[1] + E[1]]
    return out


def adjoint_image(y, f, g: Geometry, ws, exact: bool = True) -> np.ndarray:
    """``F^T y``: OlaGPU.cnvtp, F branch, olaGPU.py:261-311.

    Correlate each frame with its PSF (``IFFT(FFT(frame) * conj(FFT(f)))``,
    olaGPU.py:289-297), crop each slice to ``sw`` (olaGPU.py:305), multiply
    by the window (:306), overlap-add with extent ``sw`` and crop to ``sx``
    (:307-310).  The reference overlap-adds with extent ``sw + sf - 1`` over
    ``sw``-sized slices (an out-of-bounds read); both modes here use ``sw``.
    """
    N = g.sfft
    fr = residual_frames(y, g, exact)
    Fh = _rfft2(pad_stack(np.asarray(f, np.float64), N))
    z = _irfft2(_rfft2(fr) * np.conj(Fh), s=N)
    zs = crop_stack(z, g.sw) * ws
    return crop(ola(zs, g.csf, g.sw, g.hop), g.sx)


def adjoint_psf(y, x, g: Geometry, ws, exact: bool = True) -> np.ndarray:
    """``X^T y``: OlaGPU.cnvtp, X branch, olaGPU.py:261-302: correlate each
    frame with the windowed patch and crop to ``sf`` (olaGPU.py:300-302)."""
    N = g.sfft
    fr = residual_frames(y, g, exact)
    Xh = _rfft2(windowed_patches(x, g, ws, N))
    z = _irfft2(_rfft2(fr) * np.conj(Xh), s=N)
    return crop_stack(z, g.sf)


# --------------------------------------------------------------------------
# PSF projections
# --------------------------------------------------------------------------


def normalize(f) -> np.ndarray:
    """Per-PSF unit sum when the sum exceeds 1e-6: gputools.py:1025-1044."""
    f = np.array(f, dtype=np.float64)
    if f.ndim == 3:
        s = f.reshape(f.shape[0], -1).sum(axis=1)
        for i in range(f.shape[0]):
            if s[i] > 1e-6:
                f[i] /= s[i]
    else:
        f /= f.sum()
    return f


def cliplower(x, lb) -> np.ndarray:
    """``x = max(x, lb)``: cliplower_GPU gputools.py:478-486."""
    return np.maximum(np.asarray(x, np.float64), lb)


def clipupper(x, ub) -> np.ndarray:
    """``x = min(x, ub)``: clipupper_GPU gputools.py:489-495."""
    return np.minimum(np.asarray(x, np.float64), ub)


def clip_normalize(f) -> np.ndarray:
    """The reference's PSF constraint: non-negativity (the ``[0, inf)``
    bounds of L-BFGS-B, olaGPU.py:404-411, or ``cliplower``) followed by
    ``normalize`` (vmbd_chimney.py:133)."""
    return normalize(cliplower(f, 0.0))


def simplex_project(f) -> np.ndarray:
    """Euclidean projection of each PSF onto ``{f >= 0, sum f = 1}``
    (Duchi, Shalev-Shwartz, Singer, Chandra 2008, Fig. 1): sort descending,
    ``rho = max{j : u_j - (sum_{i<=j} u_i - 1)/j > 0}``,
    ``tau = (sum_{i<=rho} u_i - 1)/rho``, ``f <- max(f - tau, 0)``."""
    f = np.asarray(f, np.float64)
    flat = f.reshape(f.shape[0], -1)
    u = -np.sort(-flat, axis=1)
    css = np.cumsum(u, axis=1) - 1.0
    j = np.arange(1, flat.shape[1] + 1)
    cond = u - css / j > 0
    rho = flat.shape[1] - np.argmax(cond[:, ::-1], axis=1)
    tau = css[np.arange(flat.shape[0]), rho - 1] / rho
    return np.maximum(flat - tau[:, None], 0).reshape(f.shape)


def basis_project(fs, basis) -> np.ndarray:
    """``w[b] = <fs, basis_b>``: what ``projection`` (projection.cu:3-27,
    via project_on_basis_gpu gputools.py:1184-1202) is meant to compute.  The
    kernel itself returns before a barrier and indexes the basis by the
    block-local column; this is the intended dot product."""
    fs = np.asarray(fs, np.float64).ravel()
    basis = np.asarray(basis, np.float64).reshape(len(basis), -1)
    return basis @ fs


def edgetaper(x, sf) -> np.ndarray:
    """Border taper by half Bartlett-Hann windows: edgetaper_gpu
    gputools.py:643-673 with edgetaper.cu:6-31.

    ``sf`` is made odd; ``hsf = floor(sf/2)``; the 1-D tables are the first
    ``hsf`` samples of scipy's periodic window divided by the product of the
    two windows' maxima.  Row ``i < hsf0`` is scaled by ``wy[i]``, row
    ``i > ROWS-1-hsf0`` by ``wy[ROWS-1-i]``, likewise for columns with
    ``wx``.
    """
    x = np.array(x, dtype=np.float64)
    sf = np.asarray(sf, dtype=np.int64)
    sf = sf + (1 - np.mod(sf, 2))
    wx = signal.get_window("barthann", int(sf[1]))
    wy = signal.get_window("barthann", int(sf[0]))
    maxw = wx.max() * wy.max()
    hsf = sf // 2
    wx = wx[:hsf[1]] / maxw
    wy = wy[:hsf[0]] / maxw
    R, C = x.shape
    ry = np.ones(R)
    cx = np.ones(C)
    for i in range(R):
        if i < hsf[0]:
            ry[i] = wy[i]
        elif i > R - 1 - hsf[0]:
            ry[i] = wy[R - 1 - i]
    for j in range(C):
        if j < hsf[1]:
            cx[j] = wx[j]
        elif j > C - 1 - hsf[1]:
            cx[j] = wx[C - 1 - j]
    return x * ry[:, None] * cx[None, :]


# --------------------------------------------------------------------------
# Fourier-division deconvolution (OlaGPU.deconv 'xdirect' / 'direct')
# --------------------------------------------------------------------------


def psf_spectrum(f, g: Geometry) -> np.ndarray:
    """F-hat of an F object: FFT of the zero-padded PSFs (olaGPU.py:142-157),
    half spectrum (``rfft2``) of the ``sfft`` frame."""
    return _rfft2(pad_stack(np.asarray(f, np.float64), g.sfft))


def image_spectrum(x, g: Geometry, ws) -> np.ndarray:
    """X-hat of an X object: FFT of the windowed, zero-padded patches
    (olaGPU.py:147-157), half spectrum."""
    return _rfft2(windowed_patches(x, g, ws, g.sfft))


def laplacian_spectrum(sz) -> np.ndarray:
    """``L = |FFT(gx)|^2 + |FFT(gy)|^2`` of the difference filters
    ``gx = [[-1, 1]]`` and ``gy = [[-1], [1]]`` zero-padded to the frame
    (olaGPU.py:553-561): ``|e^{-2 pi i k/n} - 1|^2 = 4 sin^2(pi k/n)``, full
    ``sz`` frame."""
    k0 = np.arange(int(sz[0]))
    k1 = np.arange(int(sz[1]))
    return (4.0 * np.sin(np.pi * k0 / sz[0]) ** 2)[:, None] + (4.0 * np.sin(np.pi * k1 / sz[1]) ** 2)[None, :]


def deconv_xdirect(y, Sh, g: Geometry, ws, target: str, alpha: float = 0.0, beta: float = 0.01) -> np.ndarray:
    """OlaGPU.deconv(y, mode='xdirect'), olaGPU.py:550-609: per-patch
    regularised division in Fourier space.

    * patches of ``y``: ``chop_pad(y, offset)`` with ``offset = sf - 1``
      (valid) or ``floor(sf/2)`` (same), times the window stack placed at
      the frame origin (``pad_stack(ws)``), olaGPU.py:573-584 -- the two
      supports overlap on ``[offset, sw)``;
    * ``Z = conj(S) Y / (|S|^2 + alpha L + beta)`` with ``S`` the cached
      spectrum (F-hat of an F object, X-hat of an X object):
      comp_ola_deconv_Kernel gputools.cu:316-341; ``L`` as
      ``laplacian_spectrum`` when ``alpha > 0``, else 0;
    * inverse FFT (olaGPU.py:593-595), then ``target='psf'`` (X object):
      crop each slice to ``sf`` (:598-600); ``target='image'`` (F object):
      crop to ``sw``, overlap-add with extent ``sw`` (no window), crop to
      ``sx`` (:602-607).

    ``Sh`` is the half spectrum ``[K, N0, N1//2+1]`` (``psf_spectrum`` /
    ``image_spectrum``).  The edgetaper of ``y`` at olaGPU.py:566-567 acts
    on a copy that the chop does not read (it chops the argument ``y``), so it
    does not change the result and is not restated.
    """
    if g.mode == "valid":
        off = tuple(v - 1 for v in g.sf)
    elif g.mode == "same":
        off = tuple(v // 2 for v in g.sf)
    else:
        raise NotImplementedError("Not a valid mode!")
    N = g.sfft
    yp = chop_pad(np.asarray(y, np.float64), g.csf, g.sw, g.hop, N, off) * pad_stack(np.asarray(ws, np.float64), N)
    Yh = _rfft2(yp)
    den = np.abs(Sh) ** 2 + beta
    if alpha > 0:
        den = den + alpha * laplacian_spectrum(N)[:, : N[1] // 2 + 1]
    z = _irfft2(np.conj(Sh) * Yh / den, s=N)
    if target == "psf":
        return crop_stack(z, g.sf)
    if target != "image":
        raise ValueError("target must be 'image' or 'psf'")
    return crop(ola(crop_stack(z, g.sw), g.csf, g.sw, g.hop), g.sx)


def impad(y, sz) -> np.ndarray:
    """Replicate padding by ``sz`` with ``floor(sz/2)`` rows/columns before:
    impad kernel.cu:244-266 via impad_gpu gputools.py:884-907."""
    sz = np.asarray(sz, dtype=np.int64)
    top, left = int(sz[0] // 2), int(sz[1] // 2)
    return np.pad(np.asarray(y, np.float64), ((top, int(sz[0]) - top), (left, int(sz[1]) - left)), mode="edge")


def deconv_direct(y, Fh, g: Geometry, ws, alpha: float = 0.0, beta: float = 0.01, edgetapering: int = 1,
                  factor: int = 3) -> np.ndarray:
    """OlaGPU.deconv(y, mode='direct') of an F object, olaGPU.py:515-548:
    ``xdirect`` of ``y`` clipped at 0, divided by the ``xdirect`` of a
    constant image (edgetapered by ``2 sf`` before and after, clipped to
    [0.01, 10]) to undo the window's ripple; the border
    ``factor * sf + 1`` wide is cropped (offset ``floor((factor*sf - 1)/2)``)
    and refilled by replicate padding."""
    sf = np.asarray(g.sf, dtype=np.int64)
    u = cliplower(deconv_xdirect(y, Fh, g, ws, "image", alpha, beta), 0.0)
    const = np.ones(g.sy)
    if edgetapering == 1:
        const = edgetaper(const, 2 * sf)
    c = deconv_xdirect(const, Fh, g, ws, "image", alpha, beta)
    c = clipupper(cliplower(edgetaper(c, 2 * sf), 0.01), 10.0)
    u = u / c
    sz = np.asarray(u.shape, dtype=np.int64)
    csz = sz - factor * sf - 1
    off = np.floor((factor * sf - 1) / 2.0).astype(np.int64)
    u = crop(u, csz, off)
    return impad(u, sz - csz)


def deconv_xdirect_fp32(y, operand, g: Geometry, ws, target: str, alpha: float = 0.0,
                        beta: float = 0.01) -> np.ndarray:
    """``deconv_xdirect`` in the reference's own precision: every array
    complex64/float32 and the FFTs single precision (``scipy.fft`` on float32
    input), as pyfft computes them (olaGPU.py:155, 586-595).  ``operand`` is
    the PSF stack (``target='image'``, F object) or the image
    (``target='psf'``, X object).

    Used to state how far an FP32 pipeline can be from the FP64 result: the
    PSF estimate divides by ``|X-hat|^2``, whose dynamic range (~1e9 for a
    windowed image patch) turns FFT rounding into a relative error of a few
    1e-5, for any FP32 implementation."""
    if g.mode == "valid":
        off = tuple(v - 1 for v in g.sf)
    elif g.mode == "same":
        off = tuple(v // 2 for v in g.sf)
    else:
        raise NotImplementedError("Not a valid mode!")
    N = g.sfft
    f32 = np.float32
    wsp = pad_stack(np.asarray(ws, np.float64), N).astype(f32)
    yp = chop_pad(np.asarray(y, np.float64), g.csf, g.sw, g.hop, N, off).astype(f32) * wsp
    Yh = scipy.fft.rfft2(yp)
    if target == "image":
        Sh = scipy.fft.rfft2(pad_stack(np.asarray(operand, np.float64), N).astype(f32))
    elif target == "psf":
        Sh = scipy.fft.rfft2(chop_pad(np.asarray(operand, np.float64), g.csf, g.sw, g.hop, N).astype(f32) * wsp)
    else:
        raise ValueError("target must be 'image' or 'psf'")
    den = (Sh.real * Sh.real + Sh.imag * Sh.imag).astype(f32) + f32(beta)
    if alpha > 0:
        den = den + f32(alpha) * laplacian_spectrum(N)[:, : N[1] // 2 + 1].astype(f32)
    z = scipy.fft.irfft2((np.conj(Sh) * Yh / den).astype(np.complex64), s=N)
    if target == "psf":
        return crop_stack(z, g.sf)
    return crop(ola(crop_stack(z, g.sw), g.csf, g.sw, g.hop), g.sx)
