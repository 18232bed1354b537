"""The optGPU call surface (optGPU.py) and OlaGPU's L-BFGS-B deconvolution
(olaGPU.py:315-412, 756-811) on the EFF kernels.

* ``Solopt`` -- the options structure (optGPU.py:56-127).
* ``PBB`` -- projected Barzilai-Borwein for min f(x) s.t. x >= 0 with the
  reference's reverse-communication interface (``objective.compute_obj`` /
  ``compute_grad``), on device tensors (optGPU.py:134-358).
* ``CNV_Objective`` -- 0.5||Z u - y||^2 for an ``OlaGPU`` Z (optGPU.py:33-46);
  objective and gradient come from one fused forward + adjoint pass.
* ``deconv_lbfgsb`` -- OlaGPU.deconv(mode='lbfgsb'): scipy's L-BFGS-B on the
  host with bounds [0, inf), objective 0.5||y - Z u||^2 + 0.5 beta ||u||^2,
  each evaluation one device pass (one host->device copy of u and one
  device->host copy of the objective and gradient).
"""
from __future__ import annotations

import numpy as np
import torch


class Solopt:
    """Options of PBB (optGPU.py:56-127); same names and defaults."""

    def __init__(self):
        self.maxiter = 200
        self.maxtime = 100
        self.maxmem = 10
        self.time_limit = 0
        self.use_tolx = 0
        self.use_tolo = 1
        self.use_tolg = 0
        self.use_kkt = 0
        self.tolx = 1e-8
        self.tolo = 1e-6
        self.tolk = 1e-8
        self.tolg = 1e-8
        self.verbose = 0
        self.tau = 1e-5
        self.compute_obj = 1
        self.compute_both = 0
        self.asgui = 0
        self.max_func_evals = 10
        self.pbb_gradient_norm = 1e-9
        self.beta = 0.0498
        self.sigma = 0.298
        self.unconstrained = False


class CNV_Objective:
    """0.5 ||Z u - y||^2 for an OlaGPU object Z (optGPU.py:33-46).  Both
    methods and ``compute_both`` share one fused device pass per point."""

    def __init__(self, Z, y):
        self.Z = Z
        self.y = y if isinstance(y, torch.Tensor) else torch.from_numpy(np.asarray(y, np.float32)).to(Z.device)
        self._last = None

    def compute_both(self, u):
        obj, grad = self.Z.objective(u, self.y)
        self._last = (u.data_ptr(), u._version, obj, grad)
        return obj, grad

    def _cached(self, u):
        if self._last is not None and self._last[0] == u.data_ptr() and self._last[1] == u._version:
            return self._last[2], self._last[3]
        return self.compute_both(u)

    def compute_obj(self, u):
        return self._cached(u)[0]

    def compute_grad(self, u):
        return self._cached(u)[1]


class PBB:
    """Projected Barzilai-Borwein, min f(x) s.t. x >= 0 (optGPU.py:134-358).

    Same iteration as the reference: dx = x - x_old, dg = g - g_old with the
    active bound set cleared (clip2bound, optGPU.py:129-132), step
    <dx,dx>/(1e-5 + <dx,dg>) on even and <dx,dg>/(1e-5 + <dg,dg>) on odd
    iterations (optGPU.py:222-226), x = max(x - step g, 0).  The step sizes
    are read back to the host each iteration, as in the reference.
    """

    def __init__(self, objective, x_init, options: Solopt, seed: int = 0):
        self.objective = objective
        self.options = options
        self.iter = 0
        self.status = "Failure"
        self.term_reason = 0
        self._initialisation(x_init, seed)
        if float(torch.sqrt(torch.sum(self.x * self.x))) < 1e-12:
            raise IOError("Initial vector close to zero. Cannot proceed")
        for _ in range(options.maxiter):
            self.iter += 1
            dx = self.x - self.oldx
            dg = self.g - self.oldg
            if not options.unconstrained:
                active = (self.x == 0) & (self.g > 0)
                dx = torch.where(active, torch.zeros_like(dx), dx)
                dg = torch.where(active, torch.zeros_like(dg), dg)
            self.dx, self.dg = dx, dg
            self._check_termination()
            if self.term_reason:
                break
            self.oldx, self.oldg = self.x, self.g
            if self.iter % 2 == 0:
                step = float(torch.sum(dx * dx) / (0.00001 + torch.sum(dx * dg)))
            else:
                step = float(torch.sum(dx * dg) / (0.00001 + torch.sum(dg * dg)))
            self.x = self.x - self.g * step
            if not options.unconstrained:
                self.x = self.x.clamp_min(0)
            self.oldobj = self.obj
            self.obj, self.g = objective.compute_both(self.x)
        self.status = "Success"
        self.result = self.x

    def _initialisation(self, x_init, seed):
        gen = torch.Generator(device=x_init.device).manual_seed(seed)
        y = torch.rand(x_init.shape, device=x_init.device, generator=gen)
        y = y - (x_init + 0.5)  # as the reference (optGPU.py:268)
        fx, gx = self.objective.compute_both(x_init)
        fy, gy = self.objective.compute_both(y)
        if fx < fy:
            self.x, self.oldx, self.g, self.oldg, self.obj, self.oldobj = x_init, y, gx, gy, fx, fy
        else:
            self.x, self.oldx, self.g, self.oldg, self.obj, self.oldobj = y, x_init, gy, gx, fy, fx

    def _check_termination(self):
        o = self.options
        if o.use_tolx:
            if float(torch.norm(self.dx) / torch.norm(self.oldx)) < o.tolx:
                self.term_reason = "Relative change in x small enough"
                return
        if o.use_tolo and self.iter > 2:
            if abs(self.obj - self.oldobj) < o.tolo:
                self.term_reason = "Relative change in objvalue small enough"
                return
        if self.iter >= o.maxiter:
            self.term_reason = "Maximum number of iterations reached"
            return
        self.term_reason = 0


def deconv_lbfgsb(Z, y, z0=None, maxfun=100, alpha=0.0, beta=0.01, verbose=-1, m=5):
    """OlaGPU.deconv(y, mode='lbfgsb'), olaGPU.py:381-412: minimise
    0.5||y - Z u||^2 + 0.5 beta ||u||^2 over u >= 0 with scipy's L-BFGS-B
    (the reference's factr 10 and pgtol 1e-14, bounds [0, inf)).  ``z0``
    defaults to Z^T y.  Returns (u, f(u), info) like fmin_l_bfgs_b."""
    from scipy.optimize import minimize
    if alpha > 0:
        raise NotImplementedError("the gradient (Laplacian) regulariser is not on this path")
    dev = Z.device
    yt = y if isinstance(y, torch.Tensor) else torch.from_numpy(np.asarray(y, np.float32)).to(dev)
    if tuple(yt.shape) != tuple(Z.sy):
        raise IOError("Sizes incompatible. Expected blurred image!")
    shape = Z.operand_shape
    if z0 is None:
        z0 = Z.cnvtp(yt).detach().double().cpu().numpy().ravel()
    else:
        z0 = np.asarray(z0, np.float64).ravel()
    host = torch.empty(int(np.prod(shape)), dtype=torch.float32).pin_memory()

    def fg(z):
        host.copy_(torch.from_numpy(z.astype(np.float32)))
        u = host.to(dev, non_blocking=True).view(shape)
        obj, grad = Z.objective(u, yt)
        obj = float(obj) + 0.5 * beta * float(np.dot(z, z))
        g = grad.double().cpu().numpy().ravel() + beta * z
        return obj, g

    r = minimize(fg, z0, jac=True, method="L-BFGS-B", bounds=[(0.0, None)] * z0.size,
                 options={"maxfun": maxfun, "maxcor": m, "ftol": 10.0 * np.finfo(float).eps, "gtol": 10e-15})
    if verbose > 0:
        print(f"L-BFGS-B: {r.nfev} evaluations, f = {r.fun:.6g}: {r.message}")
    info = {"grad": r.jac, "funcalls": r.nfev, "nit": r.nit, "warnflag": 0 if r.success else 1,
            "task": r.message}
    return np.reshape(r.x, shape), float(r.fun), info
