"""Online multi-frame blind deconvolution on the EFF kernels.

The frame loop of vmbd_chimney.py:110-182 (and run_vmbd.py:139-205): for
every observed frame y, estimate the spatially varying PSFs f for the current
latent image x, then update x.  The reference estimates f with L-BFGS-B
(olaGPU.py:381-412, on the host, one H2D/D2H per evaluation) and takes one
multiplicative image step; this driver runs, entirely on the device and
without host synchronisation (so a whole frame can be captured in one CUDA
graph):

1. edgetaper of y (edgetaper_gpu, gputools.py:643-673) and the saturation
   mask m = (y < 1) (vmbd_chimney.py:118);
2. ``n_pg`` projected-gradient PSF steps: g = X^T (X f - y) from the fused
   kernels, step from an exact line search on the first step and
   Barzilai-Borwein steps after it (PBB's rule, optGPU.py:222-226), Euclidean
   projection of every PSF onto the unit simplex;
3. ``n_mu`` multiplicative image steps x *= max(F^T(m y) / (F^T(m F x) + tol),
   tol), x <= max of x over the interior (vmbd_chimney.py:143-147), with
   F^T(m y) below 1e-6 of its maximum taken as 0 (FP32 transform noise where
   no data reaches a pixel; exact arithmetic gives 0 there).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .eff import EffPlan, _ptr, _stream
from .geometry import win2winaux
from .gputools import EdgeTaper, impad_gpu


class OnlineMFBD:
    # Fraction of max F^T(m y) below which it is FP32 transform noise (see
    # eff_mu_update in include/vmbd_eff.h).
    NUM_FLOOR = 1e-6

    def __init__(self, sy, sf, csf, overlap=0.5, n_pg=10, n_mu=5, tol=1e-10, taper=True,
                 device=None, sw=None, nhop=None, adjoint="exact", sfft=0, threads=0):
        self.sy = (int(sy[0]), int(sy[1]))
        self.sf = (int(sf[0]), int(sf[1]))
        self.sx = tuple(self.sy[d] + self.sf[d] - 1 for d in range(2))
        self.device = torch.device(device if device is not None else "cuda")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.winaux = win2winaux(self.sx, csf, overlap, sw=sw, nhop=nhop)
        # sfft / threads: FFT frame and CTA size of the plan (0: automatic)
        self.plan = EffPlan(self.winaux, self.sf, "valid", device=self.device, sfft=sfft, threads=threads)
        self.n_pg, self.n_mu, self.tol = int(n_pg), int(n_mu), float(tol)
        self.adjoint = adjoint
        self.lib = _lib.load()
        K = self.winaux.K
        self.n = self.sf[0] * self.sf[1]
        dev = self.device

        def z(shape, dtype=torch.float32):
            return torch.zeros(shape, dtype=dtype, device=dev)

        self.y = z(self.sy)              # current frame (static input buffer)
        self.mask = z(self.sy)
        self.x = z(self.sx)              # latent image
        self.f = torch.full((K,) + self.sf, 1.0 / self.n, device=dev)
        self.f_prev = z((K,) + self.sf)
        self.g = z((K,) + self.sf)
        self.g_prev = z((K,) + self.sf)
        self.xhat = self.plan.empty_spectrum()
        self.fhat = self.plan.empty_spectrum()
        self.ypred = z(self.sy)
        self.yg = z(self.sy)
        self.num = z(self.sx)
        nx = self.sx[0] * self.sx[1]
        # den and the interior-maximum word share one buffer, so that one
        # side job of the image forward clears both
        self._denx = z(nx + 1)
        self.den = self._denx[:nx].view(self.sx)
        self.dots = z(3, torch.float64)
        self.state = torch.ones(1, dtype=torch.float32, device=dev)
        self.xmax = self._denx[nx:].view(torch.int32)
        self.nummax = z(1, torch.int32)
        self.taper = EdgeTaper(self.sf, dev) if taper else None

    # ------------------------------------------------------------------
    def init_latent(self, frames: torch.Tensor) -> None:
        """x = replicate-padded mean of the first frames (vmbd_chimney.py:89-97)."""
        y0 = frames.reshape(-1, *self.sy).mean(0)
        self.x.copy_(impad_gpu(y0, tuple(v - 1 for v in self.sf)))

    def _check(self, s):
        _lib.check(s)

    def frame(self, y: torch.Tensor = None) -> None:
        """Process one frame (``y`` is copied into the static input buffer;
        pass None when it is already there, e.g. under graph replay)."""
        self.begin_frame(y)
        for k in range(self.n_pg):
            self.psf_step(k)
        self.begin_image_steps()
        for i in range(self.n_mu):
            self.image_step(i)

    # The frame's stages, in the order frame() runs them (each only enqueues
    # work on the current stream).  Accumulated outputs are cleared as side
    # jobs of earlier kernels that do not touch them (EFF_OUT_ZEROED on their
    # own call), so the frame graph has three clears instead of ~40.
    def begin_frame(self, y: torch.Tensor = None) -> None:
        """Edgetaper of y, the saturation mask, the X object of x."""
        if y is not None:
            self.y.copy_(y)
        if self.taper is not None:
            self.taper(self.y)
        torch.lt(self.y, 1.0, out=self.mask)  # bool -> float via out dtype
        self.plan.image_spectrum(self.x, out=self.xhat)

    def psf_step(self, k: int) -> None:
        """PSF step k: g = X^T (X f - y), step size (k = 0: exact line
        search; then BB1 / BB2 alternately), f <- P_simplex(f - s g); the
        previous f and g move to f_prev / g_prev, s to ``state``."""
        L, st, P = self.lib, _stream(self.device), self.plan
        K, n = self.winaux.K, self.n
        ny = self.sy[0] * self.sy[1]
        OZ = _lib.OUT_ZEROED
        amode = _lib.ADJ_EXACT if self.adjoint == "exact" else _lib.ADJ_REFERENCE
        # residual X f - y into y_pred (cleared by the previous PSF step;
        # cleared by the call at k = 0); side jobs: clear dots (and yg at k = 0)
        self._check(L.eff_forward_ex(P._h, _lib.OPERAND_PSF, _ptr(self.f), _ptr(self.xhat), _ptr(self.ypred),
                                     _ptr(self.y), None, OZ if k > 0 else 0, _ptr(self.yg) if k == 0 else None,
                                     ny if k == 0 else 0, _ptr(self.dots), 3, 1, st))
        # g = X^T (X f - y); the BB / exact-line-search steps need no objective value
        # (launched to overlap the forward's tail; it waits for the forward)
        self._check(L.eff_adjoint_ex(P._h, _ptr(self.ypred), None, None, None, _ptr(self.xhat),
                                     None, _ptr(self.g), None, amode, _lib.AFTER_FORWARD, 1, st))
        if k == 0:
            self._check(L.eff_forward_ex(P._h, _lib.OPERAND_PSF, _ptr(self.g), _ptr(self.xhat),
                                         _ptr(self.yg), None, None, OZ, None, 0, None, 0, 1, st))
            self._check(L.eff_dots3(_ptr(self.g), None, K * n, _ptr(self.yg), None, ny,
                                    _ptr(self.dots), OZ, st))
            mode = 0
        else:
            self._check(L.eff_dots3(_ptr(self.f), _ptr(self.f_prev), K * n, _ptr(self.g),
                                    _ptr(self.g_prev), K * n, _ptr(self.dots), OZ, st))
            mode = 1 if k % 2 == 1 else 2
        # side job: clear y_pred for the next forward
        self._check(L.eff_pg_step(_ptr(self.f), _ptr(self.g), _ptr(self.f_prev), _ptr(self.g_prev),
                                  K, n, _ptr(self.dots), mode, _ptr(self.state), _ptr(self.ypred), ny, st))

    def begin_image_steps(self) -> None:
        """F object of the new PSFs, num = F^T(m y) and its maximum."""
        L, st, P = self.lib, _stream(self.device), self.plan
        nx = self.sx[0] * self.sx[1]
        amode = _lib.ADJ_EXACT if self.adjoint == "exact" else _lib.ADJ_REFERENCE
        P.psf_spectrum(self.f, out=self.fhat)
        self._check(L.eff_adjoint_masked(P._h, _ptr(self.y), _ptr(self.mask), _ptr(self.fhat), None,
                                         _ptr(self.num), None, amode, 1, st))
        self._check(L.eff_max_nonneg(_ptr(self.num), nx, _ptr(self.nummax), st))

    def image_step(self, i: int) -> None:
        """Image step i: den = F^T(m F x), x *= max(num / (den + tol), tol),
        x <= max of x over the interior."""
        L, st, P = self.lib, _stream(self.device), self.plan
        ny = self.sy[0] * self.sy[1]
        OZ, nx = _lib.OUT_ZEROED, self.sx[0] * self.sx[1]
        amode = _lib.ADJ_EXACT if self.adjoint == "exact" else _lib.ADJ_REFERENCE
        # y_pred = F x (y_pred cleared by the previous PSF step or image
        # step); side job: clear den and the interior-maximum word
        self._check(L.eff_forward_ex(P._h, _lib.OPERAND_IMAGE, _ptr(self.x), _ptr(self.fhat),
                                     _ptr(self.ypred), None, None, OZ if (i > 0 or self.n_pg > 0) else 0,
                                     _ptr(self._denx), nx + 1, None, 0, 1, st))
        self._check(L.eff_adjoint_ex(P._h, _ptr(self.ypred), None, _ptr(self.mask), _ptr(self.fhat), None,
                                     _ptr(self.den), None, None, amode, OZ | _lib.AFTER_FORWARD, 1, st))
        last = i == self.n_mu - 1
        self._check(L.eff_mu_update(_ptr(self.x), _ptr(self.num), _ptr(self.den),
                                    ctypes.c_float(self.tol), self.sx[0], self.sx[1], self.sf[0],
                                    self.sf[1], _ptr(self.nummax), ctypes.c_float(self.NUM_FLOOR),
                                    _ptr(self.xmax), OZ, None if last else _ptr(self.ypred),
                                    0 if last else ny, st))

    def launches_per_frame(self) -> int:
        """Kernels of this library one frame launches (the two clears, of
        the first forward's output and of the masked adjoint's, included)."""
        return ((1 if self.taper else 0) + 1 + self.n_pg * 4 + 1 + 1 + 1 + 1 + self.n_mu * 4 + 2)


def make_sequence(plan: EffPlan, n_frames: int, seed: int = 3, peak: float = 1000.0, sigma: float = 0.005):
    """Synthetic online-MFBD data: one latent blob+edge image of the plan's
    image size, per-frame PSFs drifting smoothly (random-walk motion blur),
    y_t = EFF(x, f_t) with Poisson noise at ``peak`` photons plus Gaussian
    noise of std ``sigma``.  Returns (x_true, f_seq, y_seq) on the device."""
    from .synth import blob_edge_image, drifting_motion_psfs
    dev = plan.device
    x = torch.from_numpy(blob_edge_image(plan.sx, seed=seed)).to(dev)
    f = torch.from_numpy(drifting_motion_psfs(n_frames, plan.K, plan.sf, seed=seed + 1)).to(dev)
    gen = torch.Generator(device=dev).manual_seed(seed + 2)
    ys = torch.empty((n_frames,) + plan.sy, device=dev)
    for t in range(n_frames):
        clean = plan.forward_both(x, f[t]).clamp_(min=0)
        noisy = torch.poisson(clean * peak, generator=gen) / peak
        ys[t] = noisy + sigma * torch.randn(plan.sy, device=dev, generator=gen)
    return x, f, ys
