"""GPU: the online MFBD step (edgetaper, projected-gradient PSF steps, the
multiplicative image step) against the FP64 oracle of the same frame loop."""
import ctypes

import numpy as np
import pytest

from oracle import eff64, mfbd64

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_edgetaper_matches_reference_restatement(cuda):
    import torch
    from vmbd_gb300.gputools import edgetaper_gpu
    rng = np.random.default_rng(0)
    for shape, sf in (((64, 80), (9, 12)), ((512, 512), (25, 25))):
        y = rng.random(shape).astype(np.float32)
        out = edgetaper_gpu(torch.from_numpy(y).to(cuda), sf).cpu().numpy()
        assert np.abs(out - eff64.edgetaper(y, sf)).max() < 1e-6


def test_pg_step_and_dots(cuda):
    import torch
    from vmbd_gb300 import _lib
    from vmbd_gb300.eff import _ptr
    from vmbd_gb300.gputools import dots3
    lib = _lib.load()
    rng = np.random.default_rng(1)
    K, sf = 16, (25, 25)
    n = sf[0] * sf[1]
    f = eff64.simplex_project(rng.random((K,) + sf))
    fp = eff64.simplex_project(rng.random((K,) + sf))
    g = rng.standard_normal((K,) + sf) * 1e-3
    gp = g + rng.standard_normal((K,) + sf) * 1e-4
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(cuda)
    ft, fpt, gt, gpt = t(f), t(fp), t(g), t(gp)
    d = dots3(ft, gt, fpt, gpt).cpu().numpy()
    f32, fp32, g32, gp32 = (a.astype(np.float32).astype(np.float64) for a in (f, fp, g, gp))
    dx, dg = f32 - fp32, g32 - gp32
    ref = np.array([np.sum(dx * dx), np.sum(dx * dg), np.sum(dg * dg)])
    assert np.allclose(d, ref, rtol=1e-5)
    for mode in (1, 2):
        state = torch.ones(1, device=cuda)
        dd = torch.from_numpy(ref).to(cuda)
        f2, g2, fp2, gp2 = t(f), t(g), t(fp), t(gp)
        side = torch.ones(70001, device=cuda)  # cleared as the step's side job
        _lib.check(lib.eff_pg_step(_ptr(f2), _ptr(g2), _ptr(fp2), _ptr(gp2), K, n, _ptr(dd), mode,
                                   _ptr(state), _ptr(side), side.numel(), None))
        assert not side.any()
        s = mfbd64.step_size(ref, mode, 1.0)
        want = eff64.simplex_project(f32 - s * g32)
        assert abs(float(state) - s) < 1e-6 * s
        assert np.abs(f2.cpu().numpy() - want).max() < 2e-6
        assert np.array_equal(fp2.cpu().numpy(), f.astype(np.float32))
        assert np.array_equal(gp2.cpu().numpy(), g.astype(np.float32))


def small_problem(cuda, n_frames=2):
    from vmbd_gb300.mfbd import OnlineMFBD, make_sequence
    M = OnlineMFBD((100, 116), (9, 9), (3, 3), n_pg=10, n_mu=5, device=cuda)
    _, _, ys = make_sequence(M.plan, n_frames, seed=4)
    M.init_latent(ys[:1])
    return M, ys


def test_mfbd_frames_match_fp64_oracle(cuda):
    M, ys = small_problem(cuda)
    g = eff64.Geometry(M.sx, M.sf, M.winaux.csf, M.winaux.sw, M.winaux.nhop, "valid")
    ws = M.winaux.ws.astype(np.float64)
    x = M.x.cpu().numpy().astype(np.float64)
    f = M.f.cpu().numpy().astype(np.float64)
    state = 1.0
    for t in range(ys.shape[0]):
        y = ys[t].cpu().numpy()
        M.frame(ys[t])
        extra = {}
        x, f, state, objs = mfbd64.mfbd_frame(x, f, y, g, ws, state=state, out=extra)
        xg, fg = M.x.cpu().numpy(), M.f.cpu().numpy()
        # An iterative solve: per-op rounding (1e-7) propagated through 15
        # steps.  The image step is compared where data reaches the pixel
        # (numerator above 1e-4 of its max); on the few border pixels next
        # to the FP32 noise floor the update is ill-conditioned in any
        # precision, so there only the common bound is checked.
        num = extra["num"]
        sup = num > 1e-4 * num.max()
        assert sup.mean() > 0.9
        assert rel(xg[sup], x[sup]) < 1e-3, t
        assert xg.max() <= x.max() * (1 + 1e-3) + 1e-6
        assert rel(fg, f) < 1e-3, t
        assert np.allclose(fg.reshape(fg.shape[0], -1).sum(1), 1, atol=1e-5)
        assert fg.min() >= 0 and xg.min() >= 0
        assert objs[-1] < objs[0]


def test_mfbd_frame_graph_replay_matches_eager(cuda):
    import torch
    M, ys = small_problem(cuda, n_frames=2)
    M2, _ = small_problem(cuda, n_frames=1)
    M2.x.copy_(M.x)
    M2.f.copy_(M.f)
    M.frame(ys[0])  # eager
    stream = torch.cuda.Stream(device=cuda)
    M2.y.copy_(ys[0])
    torch.cuda.synchronize(cuda)
    with torch.cuda.stream(stream):
        M2.frame(None)  # warm-up (first use of every kernel) on the capture stream
        torch.cuda.synchronize(cuda)
        gph = torch.cuda.CUDAGraph()
        # reset to the pre-frame state, then capture one frame
        M2.x.copy_(M.x)
        with torch.cuda.graph(gph, stream=stream):
            M2.frame(None)
    torch.cuda.synchronize(cuda)
    # replay from the same starting point as the eager run
    M3, _ = small_problem(cuda, n_frames=1)
    M2.x.copy_(M3.x)
    M2.f.copy_(M3.f)
    M2.state.fill_(1.0)
    M2.y.copy_(ys[0])
    gph.replay()
    torch.cuda.synchronize(cuda)
    assert rel(M2.x.cpu().numpy(), M.x.cpu().numpy()) < 1e-4
    assert rel(M2.f.cpu().numpy(), M.f.cpu().numpy()) < 1e-4
