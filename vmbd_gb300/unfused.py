"""Unfused per-stage GPU comparator: the reference's stage sequence on torch.

Not the product path -- this is the baseline the fused kernels are measured
against.  It follows OlaGPU.cnv / cnvtp (olaGPU.py:170-311) stage by stage,
one torch op (or cuFFT call via ``torch.fft``) per stage, each stage's complex
patch stack round-tripping through HBM, with buffers preallocated by torch's
caching allocator and no per-call module loads:

forward: chop+pad (gather) -> window multiply -> FFT -> spectral multiply ->
inverse FFT -> overlap-add (``F.fold``) -> crop.
adjoints: chop+pad of y -> FFT -> two spectral products -> two inverse FFTs
-> crop to sw, window, overlap-add, crop (image) / crop to sf (PSF).
Adjoints here are exact (full-extent chop), like the fused path's default.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F

from .geometry import Winaux


class UnfusedEff:
    def __init__(self, winaux: Winaux, sf, mode="valid", N=None, device="cuda"):
        self.wa = winaux
        self.sf = tuple(int(v) for v in sf)
        self.sx = winaux.sx
        self.sw = winaux.sw
        self.hop = winaux.nhop
        self.csf = winaux.csf
        self.K = winaux.K
        E = tuple(self.sw[d] + self.sf[d] - 1 for d in range(2))
        self.E = E
        n = 64
        while n < max(E):
            n *= 2
        self.N = N or n
        self.mode = mode
        self.off = {"valid": tuple(v - 1 for v in self.sf), "same": tuple(v // 2 for v in self.sf),
                    "full": (0, 0)}[mode]
        self.sy = {"valid": tuple(self.sx[d] - self.sf[d] + 1 for d in range(2)), "same": self.sx,
                   "full": tuple(self.sx[d] + self.sf[d] - 1 for d in range(2))}[mode]
        self.sxp = winaux.sxp
        self.full = tuple(self.sxp[d] + self.sf[d] - 1 for d in range(2))
        dev = torch.device(device)
        self.ws = torch.from_numpy(winaux.ws).to(dev)
        # gather index of patch k's sw window in the zero-padded image
        ii = torch.arange(self.csf[0], device=dev)[:, None] * self.hop[0] + torch.arange(self.sw[0], device=dev)
        jj = torch.arange(self.csf[1], device=dev)[:, None] * self.hop[1] + torch.arange(self.sw[1], device=dev)
        self.ii, self.jj = ii, jj
        # frames of the output-side image for the exact adjoint (extent E)
        ie = torch.arange(self.csf[0], device=dev)[:, None] * self.hop[0] + torch.arange(E[0], device=dev)
        je = torch.arange(self.csf[1], device=dev)[:, None] * self.hop[1] + torch.arange(E[1], device=dev)
        self.ie, self.je = ie, je

    def _chop(self, img, ii, jj, ext):
        """[H, W] -> [K, len(ii), len(jj)] gather (zero outside the image);
        ``ext`` is the patch extent the indices cover."""
        H = max(self.hop[0] * (self.csf[0] - 1) + ext[0], img.shape[0])
        W = max(self.hop[1] * (self.csf[1] - 1) + ext[1], img.shape[1])
        p = F.pad(img, (0, W - img.shape[1], 0, H - img.shape[0]))
        pt = p[ii[:, None, :, None], jj[None, :, None, :]]  # [cm, cn, a, b]
        return pt.reshape(self.K, ii.shape[1], jj.shape[1])

    def _ola(self, stack, ext, size):
        """Overlap-add [K, ext0, ext1] patches at hop spacing -> size."""
        cols = stack.reshape(self.K, ext[0] * ext[1]).t().unsqueeze(0)
        out_sz = tuple(self.hop[d] * (self.csf[d] - 1) + ext[d] for d in range(2))
        o = F.fold(cols, out_sz, ext, stride=self.hop)[0, 0]
        return o[:size[0], :size[1]] if o.shape[0] >= size[0] and o.shape[1] >= size[1] else \
            F.pad(o, (0, max(0, size[1] - o.shape[1]), 0, max(0, size[0] - o.shape[0])))[:size[0], :size[1]]

    def psf_spectrum(self, f):
        N = self.N
        fp = F.pad(f, (0, N - self.sf[1], 0, N - self.sf[0]))
        return torch.fft.fft2(fp.to(torch.complex64))

    def image_spectrum(self, x):
        N = self.N
        u = self._chop(x, self.ii, self.jj, self.sw) * self.ws
        u = F.pad(u, (0, N - self.sw[1], 0, N - self.sw[0]))
        return torch.fft.fft2(u.to(torch.complex64))

    def forward(self, x, fhat):
        xh = self.image_spectrum(x)
        ys = torch.fft.ifft2(fhat * xh)
        yre = ys.real[:, :self.E[0], :self.E[1]].contiguous()
        yfull = self._ola(yre, self.E, self.full)
        o = self.off
        out = torch.zeros(self.sy, device=x.device, dtype=torch.float32)
        h = min(self.sy[0], self.full[0] - o[0])
        w = min(self.sy[1], self.full[1] - o[1])
        out[:h, :w] = yfull[o[0]:o[0] + h, o[1]:o[1] + w]
        return out, xh

    def adjoint(self, y, fhat, xhat):
        N = self.N
        o = self.off
        emb = torch.zeros(self.full, device=y.device, dtype=torch.float32)
        h = min(self.sy[0], self.full[0] - o[0])
        w = min(self.sy[1], self.full[1] - o[1])
        emb[o[0]:o[0] + h, o[1]:o[1] + w] = y[:h, :w]
        fr = self._chop(emb, self.ie, self.je, self.E)
        fr = F.pad(fr, (0, N - self.E[1], 0, N - self.E[0]))
        yh = torch.fft.fft2(fr.to(torch.complex64))
        zx = torch.fft.ifft2(yh * fhat.conj()).real[:, :self.sw[0], :self.sw[1]] * self.ws
        gx = self._ola(zx.contiguous(), self.sw, self.sx)
        zf = torch.fft.ifft2(yh * xhat.conj()).real[:, :self.sf[0], :self.sf[1]].contiguous()
        return gx, zf

    def xdirect(self, y, fhat=None, xhat=None, alpha=0.0, beta=0.01):
        """OlaGPU.deconv 'xdirect' (olaGPU.py:550-609) stage by stage: chop of
        y at frame offset ``off`` times the window at the frame origin -> FFT
        -> regularised division (one elementwise pass per stage) -> inverse
        FFT -> crop to sw + overlap-add (image) / crop to sf (PSFs)."""
        N = self.N
        o = self.off
        emb = F.pad(y, (o[1], 0, o[0], 0))
        u = self._chop(emb, self.ii, self.jj, self.sw) * self.ws
        u = F.pad(u, (0, N - self.sw[1], 0, N - self.sw[0]))
        yh = torch.fft.fft2(u.to(torch.complex64))
        reg = beta
        if alpha > 0:
            k = torch.arange(N, device=y.device, dtype=torch.float64)
            lap = (4.0 * torch.sin(torch.pi * k / N) ** 2).to(torch.float32)
            reg = alpha * (lap[:, None] + lap[None, :]) + beta
        img = psf = None
        if fhat is not None:
            z = torch.fft.ifft2(fhat.conj() * yh / (fhat.abs() ** 2 + reg)).real[:, :self.sw[0], :self.sw[1]]
            img = self._ola(z.contiguous(), self.sw, self.sx)
        if xhat is not None:
            z = torch.fft.ifft2(xhat.conj() * yh / (xhat.abs() ** 2 + reg)).real
            psf = z[:, :self.sf[0], :self.sf[1]].contiguous()
        return img, psf

    # -- pieces used by the unfused MFBD comparator ---------------------------
    def forward_from_spectra(self, xh, fh):
        ys = torch.fft.ifft2(fh * xh)
        yre = ys.real[:, :self.E[0], :self.E[1]].contiguous()
        yfull = self._ola(yre, self.E, self.full)
        o = self.off
        out = torch.zeros(self.sy, device=xh.device, dtype=torch.float32)
        h = min(self.sy[0], self.full[0] - o[0])
        w = min(self.sy[1], self.full[1] - o[1])
        out[:h, :w] = yfull[o[0]:o[0] + h, o[1]:o[1] + w]
        return out

    def frames_spectrum(self, y):
        N = self.N
        o = self.off
        emb = torch.zeros(self.full, device=y.device, dtype=torch.float32)
        h = min(self.sy[0], self.full[0] - o[0])
        w = min(self.sy[1], self.full[1] - o[1])
        emb[o[0]:o[0] + h, o[1]:o[1] + w] = y[:h, :w]
        fr = self._chop(emb, self.ie, self.je, self.E)
        fr = F.pad(fr, (0, N - self.E[1], 0, N - self.E[0]))
        return torch.fft.fft2(fr.to(torch.complex64))

    def adjoint_image_only(self, yh, fhat):
        zx = torch.fft.ifft2(yh * fhat.conj()).real[:, :self.sw[0], :self.sw[1]] * self.ws
        return self._ola(zx.contiguous(), self.sw, self.sx)

    def adjoint_psf_only(self, yh, xhat):
        return torch.fft.ifft2(yh * xhat.conj()).real[:, :self.sf[0], :self.sf[1]].contiguous()


def simplex_project_torch(v):
    """Euclidean projection of each row of v [K, n] onto the unit simplex
    (Duchi et al. 2008, sort-based)."""
    K, n = v.shape
    u, _ = torch.sort(v, dim=1, descending=True)
    css = torch.cumsum(u, 1) - 1
    j = torch.arange(1, n + 1, device=v.device, dtype=v.dtype)
    cond = (u - css / j) > 0
    rho = (cond.to(v.dtype) * j).amax(1)
    tau = css.gather(1, (rho.long() - 1).clamp_min(0)[:, None])[:, 0] / rho
    return (v - tau[:, None]).clamp_min(0)


class UnfusedMFBD:
    """The same frame loop as ``vmbd_gb300.mfbd.OnlineMFBD`` built from the
    unfused per-stage operator and plain torch ops (comparator only)."""

    def __init__(self, mfbd):
        self.m = mfbd
        self.U = UnfusedEff(mfbd.winaux, mfbd.sf, N=mfbd.plan.N, device=mfbd.device)
        from .gputools import edgetaper_tables
        wy, wx = edgetaper_tables(mfbd.sf)
        R, C = mfbd.sy
        ry = torch.ones(R, device=mfbd.device)
        cx = torch.ones(C, device=mfbd.device)
        hy, hx = len(wy), len(wx)
        ry[:hy] = torch.from_numpy(wy).to(mfbd.device)
        ry[R - hy:] = torch.from_numpy(wy[::-1].copy()).to(mfbd.device)
        cx[:hx] = torch.from_numpy(wx).to(mfbd.device)
        cx[C - hx:] = torch.from_numpy(wx[::-1].copy()).to(mfbd.device)
        self.taper = ry[:, None] * cx[None, :]
        self.state = torch.ones((), device=mfbd.device)

    def frame(self, y, x, f):
        m, U = self.m, self.U
        K, n = m.winaux.K, m.n
        y = y * self.taper
        mask = (y < 1).float()
        xh = U.image_spectrum(x)
        yh_obs = None
        fp = gp = None
        for k in range(m.n_pg):
            fh = U.psf_spectrum(f)
            yp = U.forward_from_spectra(xh, fh)
            g = U.adjoint_psf_only(U.frames_spectrum(yp - y), xh)
            if k == 0:
                xg = U.forward_from_spectra(xh, U.psf_spectrum(g))
                s = (g * g).sum() / (xg * xg).sum()
            else:
                dx, dg = (f - fp).flatten(), (g - gp).flatten()
                a, b, c = (dx * dx).sum(), (dx * dg).sum(), (dg * dg).sum()
                cand = a / b if k % 2 == 1 else b / c
                s = torch.where((b > 0) & torch.isfinite(cand) & (cand > 0), cand, self.state)
            self.state = s
            fp, gp = f, g
            f = simplex_project_torch((f - s * g).reshape(K, n)).reshape(f.shape)
        fh = U.psf_spectrum(f)
        num = U.adjoint_image_only(U.frames_spectrum(mask * y), fh)
        s0, s1 = m.sf
        for _ in range(m.n_mu):
            yp = U.forward_from_spectra(U.image_spectrum(x), fh)
            den = U.adjoint_image_only(U.frames_spectrum(mask * yp), fh)
            x = x * torch.clamp_min(num / (den + m.tol), m.tol)
            x = torch.minimum(x, x[s0:x.shape[0] - s0, s1:x.shape[1] - s1].max())
        return x, f
