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


# ---------------------------------------------------------------------------
# The online MFBD workload's geometry (512x512 frames, 8x8 grid of win2winaux
# 120x120 patches at hop 60, 25x25 drifting motion PSFs, frame 256), three
# frames, every step checked against the FP64 oracle applied to the GPU's own
# state before that step.  Each kernel output of a step must match the oracle
# at relative L2 1e-5; composite quantities (the gradient of a near-converged
# residual, the BB step size, the updated PSFs and image) get a tolerance
# derived in the step from the measured input errors and the conditioning of
# that step, instead of a blanket bound for the iteration.
# ---------------------------------------------------------------------------
EPS_FWD = 2e-7   # FP32 forward's relative L2 error bound (measured ~1e-7)
EPS_OP = 1e-6    # FP32 transform rounding of an operator, relative to |operator| |input|
EPS_PIX = 1e-6   # FP32 transform rounding, absolute, relative to an output's max


def _operator_norm(x, g, ws, sf, K, iters=8, seed=0):
    """Largest singular value of f -> EFF(x, f) (power iteration on X^T X,
    FP64 oracle)."""
    v = np.random.default_rng(seed).standard_normal((K,) + tuple(sf))
    lam = 0.0
    for _ in range(iters):
        v /= np.linalg.norm(v)
        w = eff64.adjoint_psf(eff64.forward(x, v, g, ws), x, g, ws)
        lam = float(np.sum(v * w))
        v = w
    return np.sqrt(lam)


def _h(t):
    return t.detach().double().cpu().numpy()


def _norm(a):
    return float(np.linalg.norm(a))


def test_mfbd_workload_steps_match_fp64_oracle(cuda):
    import torch
    from vmbd_gb300.mfbd import OnlineMFBD, make_sequence

    M = OnlineMFBD((512, 512), (25, 25), (8, 8), n_pg=10, n_mu=5, device=cuda)
    assert M.plan.N == 256 and M.winaux.sw == (120, 120)
    _, _, ys = make_sequence(M.plan, 3, seed=11)
    M.init_latent(ys[:1])
    g = eff64.Geometry(M.sx, M.sf, M.winaux.csf, M.winaux.sw, M.winaux.nhop, "valid")
    ws = M.winaux.ws.astype(np.float64)
    s0, s1 = M.sf
    worst = {"g": 0.0, "num": 0.0, "den": 0.0}
    for t in range(ys.shape[0]):
        M.begin_frame(ys[t])
        torch.cuda.synchronize(cuda)
        assert np.abs(_h(M.y) - eff64.edgetaper(ys[t].cpu().numpy(), M.sf)).max() < 1e-6
        y = _h(M.y)                         # the tapered frame the GPU works on
        mask = (y < 1).astype(np.float64)
        x = _h(M.x)
        # |X|: the PSF gradient X^T r near the optimum is a small difference
        # of large terms, its FP32 error scales with |X| |r| (and |X| |yp|
        # through the forward's rounding of the residual), not with |g|
        nX = _operator_norm(x, g, ws, M.sf, M.winaux.K)
        for k in range(M.n_pg):
            f0, fp0, gp0, st0 = _h(M.f), _h(M.f_prev), _h(M.g_prev), float(M.state)
            M.psf_step(k)
            torch.cuda.synchronize(cuda)
            yp = eff64.forward(x, f0, g, ws)
            r = yp - y
            g64 = eff64.adjoint_psf(r, x, g, ws)
            # bound: |X| (forward rounding of yp + the adjoint's rounding of r) / |g|
            e_g = rel(_h(M.g), g64)
            tol_g = max(1e-5, 3 * nX * (EPS_FWD * _norm(yp) + EPS_OP * _norm(r)) / _norm(g64))
            assert e_g <= tol_g, (t, k, e_g, tol_g)
            worst["g"] = max(worst["g"], e_g)
            # step size from the same state; its error bound from e_g and the
            # conditioning of the dot products it divides
            ng = _norm(g64)
            if k == 0:
                xg = eff64.forward(x, g64, g, ws)
                dots = (float(np.sum(g64 * g64)), 0.0, float(np.sum(xg * xg)))
                mode, tol_s = 0, 8 * e_g + 8 * EPS_FWD
            else:
                dx, dg = f0 - fp0, g64 - gp0
                dots = (float(np.sum(dx * dx)), float(np.sum(dx * dg)), float(np.sum(dg * dg)))
                mode = 1 if k % 2 == 1 else 2
                dd = e_g * ng * _norm(dx) / max(abs(dots[1]), 1e-300)
                tol_s = 2 * (dd if mode == 1 else dd + 2 * e_g * ng / max(_norm(dg), 1e-300)) + 1e-6
            s64 = mfbd64.step_size(dots, mode, st0)
            s_gpu = float(M.state)
            assert abs(s_gpu - s64) <= tol_s * s64, (t, k, mode, s_gpu, s64, tol_s)
            # the projected step with the GPU's step size: the projection is
            # non-expansive, so its error is at most s |dg| plus FP32 rounding
            f1 = eff64.simplex_project(f0 - s_gpu * g64)
            tol_f = 2 * s_gpu * e_g * ng / _norm(f1) + 1e-6
            assert rel(_h(M.f), f1) <= tol_f, (t, k, rel(_h(M.f), f1), tol_f)
        f = _h(M.f)
        M.begin_image_steps()
        torch.cuda.synchronize(cuda)
        num64 = eff64.adjoint_image(mask * y, f, g, ws)
        e_num = rel(_h(M.num), num64)
        assert e_num <= 1e-5, (t, e_num)
        worst["num"] = max(worst["num"], e_num)
        num_g = _h(M.num)
        num_f = np.where(num_g > M.NUM_FLOOR * max(num_g.max(), 0.0), num_g, 0.0)
        num64f = np.where(num64 > M.NUM_FLOOR * max(num64.max(), 0.0), num64, 0.0)
        for i in range(M.n_mu):
            x0 = _h(M.x)
            M.image_step(i)
            torch.cuda.synchronize(cuda)
            den64 = eff64.adjoint_image(mask * eff64.forward(x0, f, g, ws), f, g, ws)
            den_g = _h(M.den)
            e_den = rel(den_g, den64)
            assert e_den <= 1e-5, (t, i, e_den)
            worst["den"] = max(worst["den"], e_den)
            # the update kernel's own arithmetic on the GPU's inputs
            xe = x0 * np.maximum(num_f / (den_g + M.tol), M.tol)
            xe = np.minimum(xe, xe[s0:xe.shape[0] - s0, s1:xe.shape[1] - s1].max())
            assert rel(_h(M.x), xe) < 1e-6, (t, i)
            # against the oracle's update of the same x0: pointwise, an FP32
            # transform leaves an absolute error of ~EPS_PIX * max on num and
            # den, so the ratio's relative error is that over num and den
            x1 = x0 * np.maximum(num64f / (den64 + M.tol), M.tol)
            x1 = np.minimum(x1, x1[s0:x1.shape[0] - s0, s1:x1.shape[1] - s1].max())
            sup = num64f > 1e-4 * num64f.max()
            assert sup.mean() > 0.9
            bound = x1 * (EPS_PIX * num64f.max() / np.maximum(num64f, 1e-300) +
                          EPS_PIX * den64.max() / np.maximum(den64, 1e-300))
            tol_x = 3 * _norm(bound[sup]) / _norm(x1[sup]) + 1e-6
            assert rel(_h(M.x)[sup], x1[sup]) <= tol_x, (t, i, rel(_h(M.x)[sup], x1[sup]), tol_x)
    print("mfbd workload per-step worst rel-L2:", worst)
