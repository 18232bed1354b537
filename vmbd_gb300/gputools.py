"""The ``gputools`` functions on the EFF path (gputools.py), on torch CUDA
tensors, backed by the library's kernels."""
from __future__ import annotations

import ctypes

import numpy as np
import torch
from scipy import signal

from . import _lib
from .eff import _ptr, _stream, project_psf


def edgetaper_tables(sf):
    """1-D tables of edgetaper_gpu (gputools.py:643-673): ``sf`` made odd,
    the first floor(sf/2) samples of scipy's periodic Bartlett-Hann window of
    length sf, divided by the product of the two windows' maxima."""
    sf = np.asarray(sf, dtype=np.int64)
    sf = sf + (1 - np.mod(sf, 2))
    wx = signal.get_window("barthann", int(sf[1]))
    wy = signal.get_window("barthann", int(sf[0]))
    maxw = wx.max() * wy.max()
    hsf = sf // 2
    return (wy[:hsf[0]] / maxw).astype(np.float32), (wx[:hsf[1]] / maxw).astype(np.float32)


class EdgeTaper:
    """``edgetaper_gpu(y, sf)`` with the tables kept on the device."""

    def __init__(self, sf, device):
        wy, wx = edgetaper_tables(sf)
        self.wy = torch.from_numpy(wy).to(device)
        self.wx = torch.from_numpy(wx).to(device)

    def __call__(self, y: torch.Tensor) -> torch.Tensor:
        if not y.is_cuda or y.dtype != torch.float32 or not y.is_contiguous():
            raise TypeError("y must be a contiguous float32 CUDA tensor")
        rows, cols = y.shape[-2], y.shape[-1]
        batch = y.numel() // (rows * cols)
        _lib.check(_lib.load().eff_edgetaper(_ptr(y), rows, cols, _ptr(self.wy), self.wy.numel(),
                                             _ptr(self.wx), self.wx.numel(), batch, _stream(y.device)))
        return y


def edgetaper_gpu(y_gpu: torch.Tensor, sf) -> torch.Tensor:
    """In-place edge taper of a device image (gputools.py:643)."""
    return EdgeTaper(sf, y_gpu.device)(y_gpu)


def normalize(f_gpu: torch.Tensor) -> torch.Tensor:
    """Per-PSF unit sum when the sum exceeds 1e-6 (gputools.py:1025-1044),
    after clipping at 0 (the bounds the reference's solver enforces)."""
    return project_psf(f_gpu, "clip_normalize")


def cliplower_GPU(x_gpu: torch.Tensor, lb) -> torch.Tensor:
    """gputools.py:478-486."""
    return x_gpu.clamp_(min=float(lb))


def clipupper_GPU(x_gpu: torch.Tensor, ub) -> torch.Tensor:
    """gputools.py:489-495."""
    return x_gpu.clamp_(max=float(ub))


def impad_gpu(y_gpu: torch.Tensor, sf) -> torch.Tensor:
    """Replicate-pad by ``sf`` with ``floor(sf/2)`` before (impad,
    kernel.cu:244-266 via gputools.py:884-907)."""
    sf = np.asarray(sf, dtype=np.int64)
    top, left = int(sf[0] // 2), int(sf[1] // 2)
    bottom, right = int(sf[0]) - top, int(sf[1]) - left
    return torch.nn.functional.pad(y_gpu[None, None], (left, right, top, bottom), mode="replicate")[0, 0]


def dots3(a, b, ap=None, bp=None):
    """(sum u^2, sum u v, sum v^2) with u = a - ap, v = b - bp, in FP64."""
    out = torch.empty(3, dtype=torch.float64, device=a.device)
    _lib.check(_lib.load().eff_dots3(_ptr(a), _ptr(ap), a.numel(), _ptr(b), _ptr(bp), b.numel(),
                                     _ptr(out), 0, _stream(a.device)))
    return out
