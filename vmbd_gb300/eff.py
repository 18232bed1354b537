"""Torch-level EFF operator: one plan per geometry, CUDA kernels via the C ABI.

``EffPlan`` wraps ``eff_plan_create`` for a ``Winaux`` + PSF size + mode and
exposes the kernels on torch CUDA tensors (float32, C order; an optional
leading batch dim runs several images of the same geometry in one launch).
Outputs and spectrum caches are allocated by torch; every kernel runs on the
current torch stream.  Spectra are complex64 tensors of shape
``[batch?, K, N/2+1, N]``.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .geometry import Winaux


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class EffPlan:
    """Plan for ``y = EFF(x, f)`` on one geometry (OlaGPU.__init__,
    olaGPU.py:95-168, without the cached spectrum)."""

    def __init__(self, winaux: Winaux, sf, mode: str = "valid", sfft: int = 0, device=None, threads: int = 0,
                 deterministic: bool = False, lib=None):
        if mode not in _lib.MODES:
            raise NotImplementedError("Not a valid mode!")
        # lib: the library to run on (default the product library; tests pass
        # the bounds-checked variant, _lib.load_debug())
        self.lib = lib if lib is not None else _lib.load()
        self.winaux = winaux
        self.sf = (int(sf[0]), int(sf[1]))
        self.sx = winaux.sx
        self.mode = mode
        self.device = torch.device(device if device is not None else "cuda", )
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        g = _lib.EffGeom()
        g.sx[:] = self.sx
        g.sf[:] = self.sf
        g.csf[:] = winaux.csf
        g.sw[:] = winaux.sw
        g.hop[:] = winaux.nhop
        g.sfft = int(sfft)
        g.threads = int(threads)
        g.mode = _lib.MODES[mode]
        # deterministic: overlap-add by a fixed-order gather (bit-identical
        # repeats; one extra kernel per overlap-added output)
        g.flags = _lib.GEOM_DETERMINISTIC if deterministic else 0
        self.deterministic = bool(deterministic)
        self._w0 = np.ascontiguousarray(winaux.win0, dtype=np.float32)
        self._w1 = np.ascontiguousarray(winaux.win1, dtype=np.float32)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            self._st(self.lib.eff_plan_create(ctypes.byref(g), self._w0.ctypes.data,
                                                self._w1.ctypes.data, ctypes.byref(h)))
        self._h = h
        n = ctypes.c_int()
        self._st(self.lib.eff_plan_frame(h, ctypes.byref(n)))
        self.N = n.value
        self.K = winaux.K
        off = {"valid": [v - 1 for v in self.sf], "same": [v // 2 for v in self.sf], "full": [0, 0]}
        self.off = tuple(off[mode])
        if mode == "valid":
            self.sy = tuple(self.sx[d] - self.sf[d] + 1 for d in range(2))
        elif mode == "same":
            self.sy = self.sx
        else:
            self.sy = tuple(self.sx[d] + self.sf[d] - 1 for d in range(2))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self.lib.eff_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    def _st(self, status: int) -> None:
        _lib.check(status, self.lib)

    def device_errors(self, clear: bool = True) -> int:
        """Error bits the plan's kernels recorded on the device (waits for
        the device; ``EFF_DEVERR_*`` of include/vmbd_eff.h)."""
        v = ctypes.c_int()
        with torch.cuda.device(self.device):
            self._st(self.lib.eff_plan_device_errors(self._h, ctypes.byref(v), int(clear)))
        return v.value

    # ------------------------------------------------------------------
    @property
    def spectrum_shape(self) -> tuple:
        return (self.K, self.N // 2 + 1, self.N)

    def empty_spectrum(self, batch=None) -> torch.Tensor:
        shape = ((batch,) if batch else ()) + self.spectrum_shape
        return torch.empty(shape, dtype=torch.complex64, device=self.device)

    def _check(self, t, shape, name):
        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise TypeError(f"{name} must be a CUDA tensor")
        if t.dtype != torch.float32:
            raise TypeError(f"{name} must be float32")
        if tuple(t.shape[-len(shape):]) != tuple(shape):
            raise IOError(f"Size missmatch: {name} has shape {tuple(t.shape)}, expected "
                          f"[..., {', '.join(map(str, shape))}]")
        extra = t.dim() - len(shape)
        if extra > 1:
            raise IOError(f"{name}: at most one batch dimension")
        if t.device != self.device:
            raise ValueError(f"{name} is on {t.device}, plan on {self.device}")
        return t.contiguous(), (t.shape[0] if extra == 1 else None)

    def _check_spec(self, s, batch, name):
        shape = ((batch,) if batch else ()) + self.spectrum_shape
        if s.dtype != torch.complex64 or tuple(s.shape) != shape or not s.is_contiguous():
            raise IOError(f"{name} must be a contiguous complex64 tensor of shape {shape}")
        return s

    # ------------------------------------------------------------------
    def psf_spectrum(self, f, out=None):
        f, b = self._check(f, (self.K,) + self.sf, "f")
        out = self.empty_spectrum(b) if out is None else self._check_spec(out, b, "out")
        self._st(self.lib.eff_psf_spectrum(self._h, _ptr(f), _ptr(out), b or 1, _stream(self.device)))
        return out

    def image_spectrum(self, x, out=None):
        x, b = self._check(x, self.sx, "x")
        out = self.empty_spectrum(b) if out is None else self._check_spec(out, b, "out")
        self._st(self.lib.eff_image_spectrum(self._h, _ptr(x), _ptr(out), b or 1, _stream(self.device)))
        return out

    def forward_image(self, x, fhat, out=None, xhat_out=None):
        """F.cnv(x): y = EFF(x, f) with f given by its spectrum."""
        x, b = self._check(x, self.sx, "x")
        self._check_spec(fhat, b, "fhat")
        if xhat_out is not None:
            self._check_spec(xhat_out, b, "xhat_out")
        if out is None:
            out = torch.empty(((b,) if b else ()) + self.sy, dtype=torch.float32, device=self.device)
        self._st(self.lib.eff_forward_image(self._h, _ptr(x), _ptr(fhat), _ptr(out), _ptr(xhat_out),
                                              b or 1, _stream(self.device)))
        return out

    def forward_psf(self, f, xhat, out=None, fhat_out=None):
        """X.cnv(f): y = EFF(x, f) with x given by its windowed-patch spectrum."""
        f, b = self._check(f, (self.K,) + self.sf, "f")
        self._check_spec(xhat, b, "xhat")
        if fhat_out is not None:
            self._check_spec(fhat_out, b, "fhat_out")
        if out is None:
            out = torch.empty(((b,) if b else ()) + self.sy, dtype=torch.float32, device=self.device)
        self._st(self.lib.eff_forward_psf(self._h, _ptr(f), _ptr(xhat), _ptr(out), _ptr(fhat_out),
                                            b or 1, _stream(self.device)))
        return out

    def forward_both(self, x, f, out=None, xhat_out=None, fhat_out=None, subtract=None):
        """y = EFF(x, f) from raw image and PSFs in one kernel; optionally
        leaves both spectra behind for a later ``adjoint``.  ``subtract``
        (an observation y_obs): returns the residual EFF(x, f) - y_obs,
        formed by the same kernel."""
        x, b = self._check(x, self.sx, "x")
        f, bf = self._check(f, (self.K,) + self.sf, "f")
        if bf != b:
            raise IOError("Size missmatch: x and f batch dims differ")
        for s_, n in ((xhat_out, "xhat_out"), (fhat_out, "fhat_out")):
            if s_ is not None:
                self._check_spec(s_, b, n)
        if out is None:
            out = torch.empty(((b,) if b else ()) + self.sy, dtype=torch.float32, device=self.device)
        if subtract is not None:
            subtract, bs = self._check(subtract, self.sy, "subtract")
            if bs != b:
                raise IOError("Size missmatch: x and subtract batch dims differ")
            self._st(self.lib.eff_forward_residual(self._h, _ptr(x), _ptr(f), _ptr(subtract), _ptr(out),
                                                     _ptr(xhat_out), _ptr(fhat_out), b or 1,
                                                     _stream(self.device)))
            return out
        self._st(self.lib.eff_forward_both(self._h, _ptr(x), _ptr(f), _ptr(out), _ptr(xhat_out),
                                             _ptr(fhat_out), b or 1, _stream(self.device)))
        return out

    def workspace(self, batch=None) -> torch.Tensor:
        """Device workspace of ``loss_grad`` (cached per batch size)."""
        key = batch or 1
        if not hasattr(self, "_ws"):
            self._ws = {}
        if key not in self._ws:
            n = self.lib.eff_loss_grad_workspace_bytes(self._h, key)
            self._ws[key] = torch.empty(n, dtype=torch.uint8, device=self.device)
        return self._ws[key]

    def loss_grad(self, x, f, y_obs, want_image=True, want_psf=True, loss=None, gx=None, gf=None):
        """``0.5*||EFF(x, f) - y_obs||^2`` and its gradients w.r.t. x and f:
        two kernels (fused forward, fused adjoints of the residual).  Returns
        ``(loss [float64], gx, gf)``."""
        x, b = self._check(x, self.sx, "x")
        f, _ = self._check(f, (self.K,) + self.sf, "f")
        y_obs, _ = self._check(y_obs, self.sy, "y_obs")
        lead = (b,) if b else ()
        if loss is None:
            loss = torch.empty(lead, dtype=torch.float64, device=self.device)
        if want_image and gx is None:
            gx = torch.empty(lead + self.sx, dtype=torch.float32, device=self.device)
        if want_psf and gf is None:
            gf = torch.empty(lead + (self.K,) + self.sf, dtype=torch.float32, device=self.device)
        gx = gx if want_image else None
        gf = gf if want_psf else None
        ws = self.workspace(b)
        self._st(self.lib.eff_loss_grad(self._h, _ptr(x), _ptr(f), _ptr(y_obs), _ptr(loss), _ptr(gx),
                                          _ptr(gf), _ptr(ws), ws.numel(), b or 1, _stream(self.device)))
        return loss, gx, gf

    def adjoint_residual(self, y, y_obs, fhat=None, xhat=None, want_image=True, want_psf=True,
                         loss=None, gx=None, gf=None, adjoint="exact", want_loss=True):
        """``adjoint(y - y_obs)`` without forming the residual; also returns
        ``0.5*||y - y_obs||^2`` (float64; None when ``want_loss`` is False,
        which skips its reduction).  Returns ``(loss, gx, gf)``."""
        return self.adjoint(y, fhat, xhat, want_image, want_psf, adjoint, gx, gf, y_obs=y_obs,
                            loss=loss, want_loss=want_loss)

    def adjoint(self, y, fhat=None, xhat=None, want_image=True, want_psf=True,
                adjoint="exact", gx=None, gf=None, y_obs=None, loss=None, want_loss=True, residual=False):
        """F.cnvtp(y) and/or X.cnvtp(y) from one transform of y.

        Returns ``(gx, gf)``; an output that is not wanted is None.
        ``adjoint``: 'exact' (transpose of the forward) or 'reference'
        (OlaGPU.cnvtp's truncated chop).  ``residual=True``: y is already a
        residual (``forward_both(..., subtract=y_obs)``); returns
        ``(loss, gx, gf)`` with loss = 0.5 * ||y||^2 (float64)."""
        if adjoint not in ("exact", "reference"):
            raise ValueError("adjoint must be 'exact' or 'reference'")
        if adjoint == "reference" and self.mode not in ("valid", "same"):
            raise NotImplementedError("Not a valid mode!")
        y, b = self._check(y, self.sy, "y")
        want_image = want_image and fhat is not None
        want_psf = want_psf and xhat is not None
        if not (want_image or want_psf):
            raise ValueError("adjoint needs fhat (image gradient) and/or xhat (PSF gradient)")
        lead = (b,) if b else ()
        if want_image:
            self._check_spec(fhat, b, "fhat")
            if gx is None:
                gx = torch.empty(lead + self.sx, dtype=torch.float32, device=self.device)
        else:
            gx = None
        if want_psf:
            self._check_spec(xhat, b, "xhat")
            if gf is None:
                gf = torch.empty(lead + (self.K,) + self.sf, dtype=torch.float32, device=self.device)
        else:
            gf = None
        mode = _lib.ADJ_EXACT if adjoint == "exact" else _lib.ADJ_REFERENCE
        if residual:
            if y_obs is not None:
                raise ValueError("residual=True takes no y_obs")
            if not want_loss:
                loss = None
            elif loss is None:
                loss = torch.empty(lead, dtype=torch.float64, device=self.device)
            self._st(self.lib.eff_adjoint_ex(self._h, _ptr(y), None, None, _ptr(fhat if want_image else None),
                                               _ptr(xhat if want_psf else None), _ptr(gx), _ptr(gf), _ptr(loss),
                                               mode, _lib.LOSS_OF_Y, b or 1, _stream(self.device)))
            return loss, gx, gf
        if y_obs is None:
            self._st(self.lib.eff_adjoint(self._h, _ptr(y), _ptr(fhat if want_image else None),
                                            _ptr(xhat if want_psf else None), _ptr(gx), _ptr(gf), mode,
                                            b or 1, _stream(self.device)))
            return gx, gf
        y_obs, _ = self._check(y_obs, self.sy, "y_obs")
        if not want_loss:
            loss = None
        elif loss is None:
            loss = torch.empty(lead, dtype=torch.float64, device=self.device)
        self._st(self.lib.eff_adjoint_residual(self._h, _ptr(y), _ptr(y_obs),
                                                 _ptr(fhat if want_image else None),
                                                 _ptr(xhat if want_psf else None), _ptr(gx), _ptr(gf),
                                                 _ptr(loss), mode, b or 1, _stream(self.device)))
        return loss, gx, gf

    def deconv_xdirect(self, y, fhat=None, xhat=None, alpha: float = 0.0, beta: float = 0.01, u=None, fz=None):
        """OlaGPU.deconv(y, mode='xdirect'), olaGPU.py:550-609: per-patch
        division ``conj(S) Y / (|S|^2 + alpha L + beta)`` in this plan's
        N x N frame.  ``fhat`` (F object) gives the image estimate ``u``
        [..., sx]; ``xhat`` (X object) the PSF estimate ``fz`` [..., K, sf].
        Returns ``(u, fz)``; an output that is not asked for is None."""
        if self.mode not in ("valid", "same"):
            raise NotImplementedError("Not a valid mode!")
        if fhat is None and xhat is None:
            raise ValueError("deconv_xdirect needs fhat (image estimate) and/or xhat (PSF estimate)")
        y, b = self._check(y, self.sy, "y")
        lead = (b,) if b else ()
        if fhat is not None:
            self._check_spec(fhat, b, "fhat")
            if u is None:
                u = torch.empty(lead + self.sx, dtype=torch.float32, device=self.device)
        if xhat is not None:
            self._check_spec(xhat, b, "xhat")
            if fz is None:
                fz = torch.empty(lead + (self.K,) + self.sf, dtype=torch.float32, device=self.device)
        self._st(self.lib.eff_deconv_xdirect(self._h, _ptr(y), _ptr(fhat), _ptr(xhat),
                                               _ptr(u if fhat is not None else None),
                                               _ptr(fz if xhat is not None else None), float(alpha),
                                               float(beta), b or 1, _stream(self.device)))
        return (u if fhat is not None else None), (fz if xhat is not None else None)


def project_psf(f: torch.Tensor, mode: str = "simplex") -> torch.Tensor:
    """In-place PSF projection of a [..., K, sf0, sf1] stack: 'simplex'
    (Euclidean projection onto the unit simplex) or 'clip_normalize' (the
    reference's non-negativity + normalize, gputools.py:1025-1044)."""
    if not f.is_cuda or f.dtype != torch.float32 or not f.is_contiguous():
        raise TypeError("f must be a contiguous float32 CUDA tensor")
    lib = _lib.load()
    m = {"simplex": _lib.PROJ_SIMPLEX, "clip_normalize": _lib.PROJ_CLIP_NORMALIZE}[mode]
    n = f.shape[-1] * f.shape[-2]
    K = f.numel() // n
    with torch.cuda.device(f.device):
        _lib.check(lib.eff_project_psf(_ptr(f), K, n, m, _stream(f.device)))
    return f


def basis_project(fs: torch.Tensor, basis: torch.Tensor) -> torch.Tensor:
    """``w[b] = <fs, basis[b]>`` (projection.cu:3-27 as intended)."""
    lib = _lib.load()
    fs = fs.contiguous()
    basis = basis.contiguous()
    n = fs.numel()
    nb = basis.shape[0]
    if basis.numel() != nb * n:
        raise IOError("Size missmatch between basis and fs")
    w = torch.empty(nb, dtype=torch.float32, device=fs.device)
    with torch.cuda.device(fs.device):
        _lib.check(lib.eff_basis_project(_ptr(fs), _ptr(basis), _ptr(w), nb, n, _stream(fs.device)))
    return w


class EffBatch:
    """Uneven batch over several plans in one persistent launch per direction
    (``eff_batch_*``).  Per class c, arrays carry a leading dim of
    ``counts[c]`` images."""

    def _st(self, status: int) -> None:
        _lib.check(status, self.lib)

    def __init__(self, plans, counts):
        if len(plans) != len(counts) or not plans:
            raise ValueError("one count per plan")
        self.lib = _lib.load()
        self.plans = list(plans)
        self.counts = [int(c) for c in counts]
        self.device = plans[0].device
        n = len(plans)
        arr = (ctypes.c_void_p * n)(*[p._h.value for p in plans])
        cnt = (ctypes.c_int * n)(*self.counts)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            self._st(self.lib.eff_batch_create(arr, cnt, n, ctypes.byref(h)))
        self._h = h
        self._work = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self.lib.eff_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def items(self) -> int:
        return self.lib.eff_batch_items(self._h)

    @staticmethod
    def _ptrs(ts):
        if ts is None:
            return None
        return (ctypes.c_void_p * len(ts))(*[t.data_ptr() if t is not None else None for t in ts])

    def _shapes(self, ts, shape_of, name):
        for p, c, t in zip(self.plans, self.counts, ts):
            want = (c,) + shape_of(p)
            if tuple(t.shape) != want or t.dtype != torch.float32 or not t.is_contiguous() or not t.is_cuda:
                raise IOError(f"{name}: expected contiguous float32 CUDA tensor {want}, got {tuple(t.shape)}")

    def forward_both(self, xs, fs, ys=None, xhats=None, fhats=None, subtracts=None):
        """Per image y = EFF(x, f); with ``subtracts`` (observations) the
        residuals EFF(x, f) - y_obs instead."""
        self._shapes(xs, lambda p: p.sx, "x")
        self._shapes(fs, lambda p: (p.K,) + p.sf, "f")
        if ys is None:
            ys = [torch.empty((c,) + p.sy, device=self.device) for p, c in zip(self.plans, self.counts)]
        if subtracts is not None:
            self._shapes(subtracts, lambda p: p.sy, "subtract")
            self._st(self.lib.eff_batch_forward_residual(
                self._h, self._ptrs(xs), self._ptrs(fs), self._ptrs(subtracts), self._ptrs(ys),
                self._ptrs(xhats), self._ptrs(fhats), _stream(self.device)))
            return ys
        self._st(self.lib.eff_batch_forward_both(self._h, self._ptrs(xs), self._ptrs(fs), self._ptrs(ys),
                                                   self._ptrs(xhats), self._ptrs(fhats), _stream(self.device)))
        return ys

    def adjoint_residual(self, ys, y_obss, fhats, xhats, gxs=None, gfs=None, losses=None):
        """Per image the adjoints of y - y_obs and 0.5 * ||y - y_obs||^2;
        ``y_obss`` None: each y is already a residual."""
        if gxs is None:
            gxs = [torch.empty((c,) + p.sx, device=self.device) for p, c in zip(self.plans, self.counts)]
        if gfs is None:
            gfs = [torch.empty((c, p.K) + p.sf, device=self.device) for p, c in zip(self.plans, self.counts)]
        if losses is None:
            losses = [torch.empty(c, dtype=torch.float64, device=self.device) for c in self.counts]
        self._st(self.lib.eff_batch_adjoint_residual(
            self._h, self._ptrs(ys), self._ptrs(y_obss), self._ptrs(fhats), self._ptrs(xhats),
            self._ptrs(gxs), self._ptrs(gfs), self._ptrs(losses), _stream(self.device)))
        return losses, gxs, gfs

    def loss_grad(self, xs, fs, y_obss, losses=None, gxs=None, gfs=None):
        """Loss and both gradients for every image: two persistent launches."""
        if self._work is None:
            self._work = ([torch.empty((c,) + p.sy, device=self.device) for p, c in zip(self.plans, self.counts)],
                          [p.empty_spectrum(c) for p, c in zip(self.plans, self.counts)],
                          [p.empty_spectrum(c) for p, c in zip(self.plans, self.counts)])
        rs, xh, fh = self._work
        self.forward_both(xs, fs, rs, xh, fh, subtracts=y_obss)
        return self.adjoint_residual(rs, None, fh, xh, gxs, gfs, losses)


def set_cluster_mode(mode: int) -> None:
    """0: per call (default); 1: one CTA per patch; 2: a 2-CTA cluster."""
    _lib.check(_lib.load().eff_set_cluster_mode(int(mode)))
