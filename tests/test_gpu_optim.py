"""GPU: OlaGPU.deconv('lbfgsb') and PBB on the fused objective/gradient."""
import numpy as np
import pytest

from oracle import eff64

pytestmark = pytest.mark.gpu


def setup(cuda):
    import torch
    from vmbd_gb300 import OlaGPU, geometry, synth
    wa = geometry.win2winaux((120, 120), (3, 3), 0.5)
    sf = (9, 9)
    x = synth.blob_edge_image(wa.sx, seed=31)
    f = synth.gaussian_psfs(wa.K, sf, seed=32)
    g = eff64.Geometry(wa.sx, sf, wa.csf, wa.sw, wa.nhop, "valid")
    y = eff64.forward(x, f, g, wa.ws.astype(np.float64)).astype(np.float32)
    X = OlaGPU(torch.from_numpy(x).to(cuda), sf, "valid", wa)
    return X, x, f, y, g, wa


def test_objective_matches_oracle(cuda):
    import torch
    X, x, f, y, g, wa = setup(cuda)
    u = np.full_like(f, 1.0 / f[0].size)
    ut = torch.from_numpy(u).to(cuda)
    obj, grad = X.objective(ut, torch.from_numpy(y).to(cuda))
    ws = wa.ws.astype(np.float64)
    res = eff64.forward(x, u, g, ws) - y
    assert abs(obj - 0.5 * np.sum(res ** 2)) < 1e-5 * 0.5 * np.sum(res ** 2)
    # the gradient kernel against the oracle adjoint of the same FP32 residual
    res32 = X.cnv(ut).double().cpu().numpy() - y
    ref = eff64.adjoint_psf(res32, x, g, ws)
    assert np.linalg.norm(grad.cpu().numpy() - ref) / np.linalg.norm(ref) < 1e-5


def test_lbfgsb_psf_estimation_recovers_psfs(cuda):
    X, x, f, y, g, wa = setup(cuda)
    u0 = np.full(f.size, 1.0 / f[0].size)
    fh, obj, info = X.deconv(y, z0=u0, maxfun=200, beta=0.0)
    start = 0.5 * np.sum((eff64.forward(x, u0.reshape(f.shape), g, wa.ws.astype(np.float64)) - y) ** 2)
    assert obj < 2e-2 * start
    assert fh.min() >= 0
    e0 = np.linalg.norm(u0.reshape(f.shape) - f) / np.linalg.norm(f)
    assert np.linalg.norm(fh - f) / np.linalg.norm(f) < 0.5 * e0


def test_pbb_decreases_objective(cuda):
    import torch
    from vmbd_gb300.optim import CNV_Objective, PBB, Solopt
    X, x, f, y, g, wa = setup(cuda)
    obj = CNV_Objective(X, y)
    u0 = torch.full(f.shape, 1.0 / f[0].size, device=cuda)
    opts = Solopt()
    opts.maxiter = 40
    p = PBB(obj, u0, opts)
    f0 = obj.compute_obj(u0)
    # the reference's step rule (1e-5 added to the BB denominators) is scale
    # dependent and slow on PSF-sized values: check descent and feasibility
    assert p.obj < f0
    assert float(p.result.min()) >= 0
    assert p.iter >= 3
