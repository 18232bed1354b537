"""FP64 NumPy restatement of one online multi-frame blind deconvolution frame.

TEST INFRASTRUCTURE ONLY (the checker for ``vmbd_gb300.mfbd``).

Follows the frame loop of vmbd_chimney.py:110-182 with the PSF solve done by
projected gradient: PBB's Barzilai-Borwein step rule (optGPU.py:222-226,
BB1 on odd, BB2 on even iterations after an exact line search on the first)
and the Euclidean simplex projection (``eff64.simplex_project``) in place of
L-BFGS-B's bounds + ``normalize``; then ``n_mu`` multiplicative image steps
(vmbd_chimney.py:143-147), with F^T(m y) below ``num_floor`` of its maximum
taken as 0 (where no data reaches a pixel it is 0 in exact arithmetic; the
FP32 kernels see transform noise there).  Adjoints are the exact transposes.
"""
from __future__ import annotations

import numpy as np

from . import eff64


def step_size(dots, mode, prev):
    """Step from (u.u, u.v, v.v): mode 0 exact line search <g,g>/||Xg||^2,
    mode 1 BB1 <dx,dx>/<dx,dg>, mode 2 BB2 <dx,dg>/<dg,dg>; a non-positive
    curvature keeps the previous step."""
    d0, d1, d2 = dots
    if mode == 0:
        s = d0 / d2 if d2 > 0 else 0.0
    elif d1 <= 0:
        s = prev
    elif mode == 1:
        s = d0 / d1
    else:
        s = d1 / d2 if d2 > 0 else prev
    if not (s > 0) or not np.isfinite(s):
        s = prev
    return s


def mfbd_frame(x, f, y, g: eff64.Geometry, ws, n_pg=10, n_mu=5, tol=1e-10, taper=True, state=1.0,
               num_floor=1e-6, out=None):
    """One frame: returns (x, f, state, psf_objective_per_iteration); when
    ``out`` is a dict it also receives the image-step numerator ``num``."""
    y = np.asarray(y, np.float64)
    if taper:
        y = eff64.edgetaper(y, g.sf)
    mask = (y < 1).astype(np.float64)
    x = np.asarray(x, np.float64).copy()
    f = np.asarray(f, np.float64).copy()
    fp = gp = None
    objs = []
    for k in range(n_pg):
        yp = eff64.forward(x, f, g, ws)
        objs.append(0.5 * np.sum((yp - y) ** 2))
        gr = eff64.adjoint_psf(yp - y, x, g, ws)
        if k == 0:
            xg = eff64.forward(x, gr, g, ws)
            dots = (np.sum(gr * gr), 0.0, np.sum(xg * xg))
            mode = 0
        else:
            dx, dg = f - fp, gr - gp
            dots = (np.sum(dx * dx), np.sum(dx * dg), np.sum(dg * dg))
            mode = 1 if k % 2 == 1 else 2
        s = step_size(dots, mode, state)
        state = s
        fp, gp = f, gr
        f = eff64.simplex_project(f - s * gr)
    objs.append(0.5 * np.sum((eff64.forward(x, f, g, ws) - y) ** 2))
    num = eff64.adjoint_image(mask * y, f, g, ws)
    # values below num_floor * max are transform noise (0 in exact arithmetic)
    num = np.where(num > num_floor * max(num.max(), 0.0), num, 0.0)
    if out is not None:
        out["num"] = num
    s0, s1 = g.sf
    for _ in range(n_mu):
        yp = eff64.forward(x, f, g, ws)
        den = eff64.adjoint_image(mask * yp, f, g, ws)
        x = x * np.maximum(num / (den + tol), tol)
        x = np.minimum(x, x[s0:x.shape[0] - s0, s1:x.shape[1] - s1].max())
    return x, f, state, objs
