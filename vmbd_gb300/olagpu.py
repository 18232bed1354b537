"""Drop-in ``OlaGPU`` (olaGPU.py:11-311): same constructor, ``cnv`` and
``cnvtp``, backed by the fused sm_103a kernels.

``OlaGPU(z, sx, mode, winaux)``: a 3-D ``z`` (PSF stack) with ``sx`` larger
than the PSFs makes an F object that caches the PSF spectrum; a 2-D ``z``
(image) with ``sx`` smaller than it (``sx`` is then the PSF size) makes an X
object that caches the windowed-patch spectrum (olaGPU.py:104-121).
``cnv(u)`` applies the operator to an image (F) or a PSF stack (X);
``cnvtp(y)`` applies its transpose.  Inputs may be numpy arrays (returned
as numpy, host copies included, olaGPU.py:254-257) or float32 CUDA tensors
(returned as tensors).  Errors follow the reference: ``IOError`` on a size
mismatch, ``NotImplementedError`` on an unsupported mode.

One addition: ``adjoint='exact'`` (default) makes ``cnvtp`` the exact
transpose of ``cnv``; ``adjoint='reference'`` reproduces the reference's
``cnvtp``, whose chop of ``y`` drops the first ``sf-1`` rows/columns of each
patch's support (olaGPU.py:276-286).
"""
from __future__ import annotations

import numpy as np
import torch

from .eff import EffPlan
from .geometry import Winaux


def _to_device(a, device):
    if isinstance(a, torch.Tensor):
        if not a.is_cuda:
            a = a.to(device)
        return a.to(torch.float32).contiguous(), False
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32))
    return t.pin_memory().to(device, non_blocking=True), True


class OlaGPU:
    def __init__(self, f, sx, mode, winaux: Winaux, adjoint: str = "exact", sfft: int = 0):
        sf = np.array(f.shape)[-2:]
        sx = np.array(sx)
        csf = winaux.csf
        if len(f.shape) == 3 and np.all(sx > sf):
            self.__id__ = "F"
            if f.shape[0] != csf[0] * csf[1]:
                raise IOError("Size missmatch between winaux and PSF size!")
        elif len(f.shape) == 2 and np.all(sx < sf):
            self.__id__ = "X"
            sf = sx
            sx = np.array(f.shape)
        else:
            raise IOError("Size missmatch")
        if tuple(int(v) for v in winaux.sx) != tuple(int(v) for v in sx):
            raise IOError("Size missmatch between winaux and image size!")
        if mode not in ("valid", "same", "full"):
            raise NotImplementedError("Not a valid mode!")
        if adjoint not in ("exact", "reference"):
            raise ValueError("adjoint must be 'exact' or 'reference'")
        self.device = f.device if isinstance(f, torch.Tensor) and f.is_cuda else \
            torch.device("cuda", torch.cuda.current_device())
        self.plan = EffPlan(winaux, tuple(int(v) for v in sf), mode, sfft=sfft, device=self.device)
        self.winaux = winaux
        self.mode = mode
        self.adjoint = adjoint
        self.sf = tuple(int(v) for v in sf)
        self.sx = tuple(int(v) for v in sx)
        self.sy = self.plan.sy
        z, _ = _to_device(f, self.device)
        if self.__id__ == "F":
            self.f, self.x = z, None
            self.fft_gpu = self.plan.psf_spectrum(z)
        else:
            self.f, self.x = None, z
            self.fft_gpu = self.plan.image_spectrum(z)

    def cnv(self, u):
        """``F x`` (F object, u = image) or ``X f`` (X object, u = PSFs)."""
        t, host = _to_device(u, self.device)
        if self.__id__ == "F":
            if t.dim() != 2:
                raise IOError("Size missmatch between winaux and image size!")
            if tuple(t.shape) != self.winaux.sx:
                raise IOError("Size missmatch between winaux and image size!")
            y = self.plan.forward_image(t, self.fft_gpu)
        else:
            if t.dim() != 3 or t.shape[0] != self.winaux.K:
                raise IOError("Size missmatch between winaux and PSF size!")
            y = self.plan.forward_psf(t, self.fft_gpu)
        return y.cpu().numpy() if host else y

    def cnvtp(self, y):
        """``F^T y`` (image-shaped) or ``X^T y`` (PSF-stack-shaped)."""
        if self.mode not in ("valid", "same"):
            raise NotImplementedError("Not a valid mode!")
        t, host = _to_device(y, self.device)
        if self.__id__ == "F":
            out, _ = self.plan.adjoint(t, fhat=self.fft_gpu, want_psf=False, adjoint=self.adjoint)
        else:
            _, out = self.plan.adjoint(t, xhat=self.fft_gpu, want_image=False, adjoint=self.adjoint)
        return out.cpu().numpy() if host else out

    # -- optimisation support ---------------------------------------------
    @property
    def operand_shape(self):
        """Shape of what ``cnv`` takes: the image (F) or the PSF stack (X)."""
        if self.__id__ == "F":
            return tuple(self.winaux.sx)
        return (self.winaux.K,) + tuple(self.sf)

    def objective(self, u: torch.Tensor, y: torch.Tensor):
        """(0.5 ||Z u - y||^2 as a float, its gradient Z^T (Z u - y)): one
        fused forward and one fused adjoint of the residual (the pair of
        cnvinv_objfun / cnvinv_gradfun, olaGPU.py:756-811, without their
        host round trips)."""
        u = u.to(torch.float32).contiguous()
        y = y.to(torch.float32).contiguous()
        if self.__id__ == "F":
            yp = self.plan.forward_image(u, self.fft_gpu)
            loss, g, _ = self.plan.adjoint_residual(yp, y, fhat=self.fft_gpu, want_psf=False,
                                                    adjoint=self.adjoint)
        else:
            yp = self.plan.forward_psf(u, self.fft_gpu)
            loss, _, g = self.plan.adjoint_residual(yp, y, xhat=self.fft_gpu, want_image=False,
                                                    adjoint=self.adjoint)
        return float(loss), g

    def deconv(self, y, z0=None, mode="lbfgsb", maxfun=100, alpha=0.0, beta=0.01, verbose=-1, m=5,
               edgetapering=1, factor=3):
        """OlaGPU.deconv (olaGPU.py:312-733) for modes

        * 'lbfgsb' (:381-412): the PSFs (X object) or the image (F object)
          minimising 0.5||y - Z u||^2 + 0.5 beta ||u||^2, u >= 0; returns
          (u, f(u), info);
        * 'xdirect' (:550-609): per-patch regularised division in Fourier
          space, conj(S) Y / (|S|^2 + alpha L + beta); returns the image
          estimate (F object) or the PSF estimates (X object);
        * 'direct' (:515-548, F object): 'xdirect' corrected by the
          'xdirect' of a constant image, border cropped and replicate-padded.

        The division depends on the FFT frame: it runs in the reference's
        frame, the power of two >= sw + sf - 1 (one per dim; a non-square one
        raises NotImplementedError).  ``edgetapering`` only changes 'direct'
        (in 'xdirect' the reference tapers a copy that its chop never reads).
        """
        t, host = _to_device(y, self.device)
        if tuple(t.shape) != tuple(self.sy):
            raise IOError("Sizes incompatible. Expected blurred image!")
        if mode == "lbfgsb":
            from .optim import deconv_lbfgsb
            return deconv_lbfgsb(self, t, z0=z0, maxfun=maxfun, alpha=alpha, beta=beta, verbose=verbose, m=m)
        if mode == "xdirect":
            out = self._xdirect(t, alpha, beta)
        elif mode == "direct":
            if self.__id__ != "F":
                raise NotImplementedError("'direct' estimates the image: use an F object")
            out = self._direct(t, alpha, beta, edgetapering, factor)
        else:
            raise NotImplementedError("Not a valid mode!")
        return out.cpu().numpy() if host else out

    def _deconv_plan(self):
        """(plan, cached spectrum) in the reference's FFT frame
        (olaGPU.py:139-141): this object's own plan when its frame is that
        one, else a second plan with the spectrum recomputed there."""
        if self.mode not in ("valid", "same"):
            raise NotImplementedError("Not a valid mode!")
        E = [self.winaux.sw[d] + self.sf[d] - 1 for d in range(2)]
        ref = [1 << int(np.ceil(np.log2(e))) for e in E]
        if ref[0] != ref[1] or ref[0] not in (64, 128, 256, 512):
            raise NotImplementedError(f"deconv: the reference frame {ref[0]}x{ref[1]} is not one of the "
                                      "square frames 64, 128, 256, 512")
        if ref[0] == self.plan.N:
            return self.plan, self.fft_gpu
        if getattr(self, "_dplan", None) is None:
            plan = EffPlan(self.winaux, self.sf, self.mode, sfft=ref[0], device=self.device)
            spec = plan.psf_spectrum(self.f) if self.__id__ == "F" else plan.image_spectrum(self.x)
            self._dplan = (plan, spec)
        return self._dplan

    def _xdirect(self, y, alpha, beta):
        plan, spec = self._deconv_plan()
        if self.__id__ == "F":
            return plan.deconv_xdirect(y, fhat=spec, alpha=alpha, beta=beta)[0]
        return plan.deconv_xdirect(y, xhat=spec, alpha=alpha, beta=beta)[1]

    def _direct(self, y, alpha, beta, edgetapering, factor):
        from .gputools import edgetaper_gpu, impad_gpu
        sf = np.asarray(self.sf, dtype=np.int64)
        u = self._xdirect(y, alpha, beta).clamp_min_(0.0)
        const = torch.ones(tuple(self.sy), dtype=torch.float32, device=self.device)
        if edgetapering == 1:
            edgetaper_gpu(const, 2 * sf)
        c = self._xdirect(const, alpha, beta)
        edgetaper_gpu(c, 2 * sf)
        c.clamp_(0.01, 10.0)
        u = u / c
        sz = np.asarray(u.shape, dtype=np.int64)
        csz = sz - factor * sf - 1
        off = np.floor((factor * sf - 1) / 2.0).astype(np.int64)
        u = u[off[0]:off[0] + csz[0], off[1]:off[1] + csz[1]].contiguous()
        return impad_gpu(u, sz - csz)
