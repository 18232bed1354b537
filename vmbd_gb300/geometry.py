"""Patch geometry and window tables: ``win2winaux`` (imagetools.py:398-454).

Computed on the host in FP64 (it runs once per geometry).  Besides the
reference's attributes (``sx, sw, csf, nhop`` and the window stack) a
``Winaux`` carries the per-dim (alpha, gamma) tables the kernels read
(format in include/vmbd_eff.h): the partition-of-unity stack
``ws = w / chop(ola(w))`` of the separable window ``w`` factors per dim,
except on the outermost rows/columns that only zero window samples reach,
where the reference's 1e-16 floor makes ``ws = 1 / (covering patches)``.
"""
from __future__ import annotations

import math

import numpy as np
from scipy import signal


def window_1d(n: int) -> np.ndarray:
    """One factor of ``imagetools.window`` (imagetools.py:332-337): scipy's
    periodic Bartlett-Hann window, symmetrised and shifted to min 0."""
    w = signal.get_window("barthann", int(n))
    w = (w + w[::-1]) / 2
    return w - w.min()


def patch_geometry(sx, csf, overlap: float = 0.5):
    """``sw`` and ``nhop`` from the image size, imagetools.py:422-436:
    ``sw = ceil(sx / (csf*(1-ov) + ov))``, grown in both dims together until
    ``sw*ov`` is integral everywhere (or back to the first guess once it
    passes twice that), ``nhop = sw - floor(sw*ov)``."""
    sx = np.asarray(sx, dtype=np.float64)
    factor = np.asarray(csf, dtype=np.float64) * (1 - overlap) + overlap
    sw = np.ceil(sx / factor)
    first = sw
    while np.any(np.floor(sw * overlap) != sw * overlap):
        sw = sw + 1
        if np.any(sw > 2 * first):
            sw = first
            break
    nhop = sw - np.floor(sw * overlap)
    return tuple(int(v) for v in sw), tuple(int(v) for v in nhop)


class Winaux:
    """Windows and geometry for ``OlaGPU`` (imagetools.win2winaux)."""

    def __init__(self, sx, csf, sw, nhop):
        self.sx = tuple(int(v) for v in sx)
        self.csf = tuple(int(v) for v in csf)
        self.sw = tuple(int(v) for v in sw)
        self.nhop = tuple(int(v) for v in nhop)
        if any(v < 1 for v in self.sw + self.nhop + self.csf):
            raise ValueError("patch size, hop and grid must be positive")
        self.win0, self.win1 = (self._table(d) for d in range(2))
        self._ws = None
        self._ws_gpu = {}

    @property
    def K(self) -> int:
        return self.csf[0] * self.csf[1]

    @property
    def sxp(self) -> tuple:
        """Extent covered by the patch grid, gputools.py:371-372."""
        return tuple(self.nhop[d] * self.csf[d] + self.sw[d] - self.nhop[d] for d in range(2))

    def _table(self, d: int) -> np.ndarray:
        a = window_1d(self.sw[d])
        a = a / a.max()
        sxp = self.sxp[d]
        total = np.zeros(sxp)
        count = np.zeros(sxp)
        reached = np.zeros(sxp, dtype=bool)
        for m in range(self.csf[d]):
            sl = slice(m * self.nhop[d], m * self.nhop[d] + self.sw[d])
            total[sl] += a
            count[sl] += 1
            reached[sl] |= a > 0
        t = np.empty((self.csf[d], self.sw[d], 2))
        for m in range(self.csf[d]):
            i = m * self.nhop[d] + np.arange(self.sw[d])
            t[m, :, 0] = np.where(reached[i], a / np.where(total[i] > 0, total[i], 1.0), -1.0)
            t[m, :, 1] = 1.0 / count[i]
        return t.astype(np.float32)

    @property
    def ws(self) -> np.ndarray:
        """Window stack [K, sw0, sw1] (float32) rebuilt from the tables."""
        if self._ws is None:
            u = self.win0.astype(np.float64)
            v = self.win1.astype(np.float64)
            ws = np.empty((self.K,) + self.sw)
            for m in range(self.csf[0]):
                for n in range(self.csf[1]):
                    a = u[m][:, None, :]
                    b = v[n][None, :, :]
                    border = (a[..., 0] < 0) | (b[..., 0] < 0)
                    ws[m * self.csf[1] + n] = np.where(border, a[..., 1] * b[..., 1],
                                                       a[..., 0] * b[..., 0])
            self._ws = ws.astype(np.float32)
        return self._ws

    def ws_gpu(self, device="cuda"):
        """Window stack as a device tensor (the reference's ``ws_gpu``)."""
        import torch
        key = str(device)
        if key not in self._ws_gpu:
            self._ws_gpu[key] = torch.from_numpy(self.ws).to(device)
        return self._ws_gpu[key]


def win2winaux(sx, csf, overlap: float = 0.5, windowfun: str = "barthann", sw=None, nhop=None) -> Winaux:
    """imagetools.win2winaux(sx, csf, overlap): geometry + windows.

    ``sw``/``nhop`` may be given to use a stated patch size (the windows are
    then those of that grid, the image may extend past it).  As in the
    reference the window is always Bartlett-Hann (``windowfun`` is accepted
    and ignored, imagetools.py:438).
    """
    if sw is None:
        sw, nhop = patch_geometry(sx, csf, overlap)
    elif nhop is None:
        nhop = tuple(int(v) - int(math.floor(int(v) * overlap)) for v in sw)
    return Winaux(sx, csf, sw, nhop)


# Frame edges with compiled kernels; the automatic choice is the smallest
# power of two that fits (192 is used only when asked for).
FRAMES = (64, 128, 192, 256, 512)
AUTO_FRAMES = (64, 128, 256, 512)


def fft_frame(sw, sf) -> int:
    """Square frame edge the kernels pick by default: the smallest of 64,
    128, 256, 512 that is >= sw + sf - 1 in both dims (the linear convolution
    then fits without wrap-around)."""
    e = max(int(sw[0]) + int(sf[0]) - 1, int(sw[1]) + int(sf[1]) - 1)
    for n in AUTO_FRAMES:
        if n >= e:
            return n
    raise ValueError(f"sw + sf - 1 = {e} exceeds the largest frame {FRAMES[-1]}")
