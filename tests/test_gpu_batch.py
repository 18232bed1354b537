"""GPU: the uneven batch in one persistent launch (eff_batch_*) and the
autotuner, against per-image launches and the FP64 oracle."""
import numpy as np
import pytest

from oracle import eff64
from vmbd_gb300 import geometry, synth

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_class(spec, count, dev, seed):
    import torch
    from vmbd_gb300.eff import EffPlan
    sx, csf, sf, kind = spec
    wa = geometry.win2winaux(sx, csf, 0.5)
    plan = EffPlan(wa, sf, "valid", device=dev)
    gen = synth.motion_psfs if kind == "motion" else synth.gaussian_psfs
    xs = np.stack([synth.blob_edge_image(sx, seed=seed + i) for i in range(count)])
    fs = np.stack([gen(wa.K, sf, seed=seed + 50 + i) for i in range(count)])
    x = torch.from_numpy(xs).to(dev)
    f = torch.from_numpy(fs).to(dev)
    y = plan.forward_both(x, f)
    y_obs = y + 0.01 * torch.randn(y.shape, device=dev, generator=torch.Generator(device=dev).manual_seed(seed))
    return plan, x, f, y_obs


SMALL = [((96, 96), (2, 2), (9, 9), "gauss"), ((80, 112), (2, 3), (7, 7), "motion"),
         ((200, 200), (3, 3), (15, 15), "motion")]
# The uneven batch workload: 256^2 / 4x4 / 15^2, 384x512 / 6x8 / 21^2, 1024^2 / 12x12 / 31^2
WORKLOAD = [((256, 256), (4, 4), (15, 15), "gauss"), ((384, 512), (6, 8), (21, 21), "motion"),
            ((1024, 1024), (12, 12), (31, 31), "motion")]


@pytest.mark.parametrize("specs,counts", [(SMALL, (2, 3, 1)), (WORKLOAD, (2, 2, 1))], ids=["small", "workload"])
def test_persistent_batch_matches_single_launches(cuda, specs, counts):
    from vmbd_gb300.eff import EffBatch
    cls = [make_class(s, c, cuda, 10 * i) for i, (s, c) in enumerate(zip(specs, counts))]
    plans = [c[0] for c in cls]
    assert len({p.N for p in plans}) >= 2  # mixed frame sizes in one launch
    B = EffBatch(plans, counts)
    assert B.items == sum(p.K * c for p, c in zip(plans, counts))
    xs, fs, yo = [c[1] for c in cls], [c[2] for c in cls], [c[3] for c in cls]
    xhs = [p.empty_spectrum(c) for p, c in zip(plans, counts)]
    fhs = [p.empty_spectrum(c) for p, c in zip(plans, counts)]
    ys = B.forward_both(xs, fs, xhats=xhs, fhats=fhs)
    losses, gxs, gfs = B.loss_grad(xs, fs, yo)
    # the adjoint of y - y_obs formed in its row loads, and the residual
    # forward; the residual is noise-sized (1e-2 of y), so FP32 rounding of y
    # (~1e-7) is ~1e-5 of it
    l2s, gx2s, gf2s = B.adjoint_residual(ys, yo, fhs, xhs)
    rs = B.forward_both(xs, fs, subtracts=yo)
    for i in range(len(cls)):
        assert rel(rs[i].cpu(), (ys[i] - yo[i]).cpu()) < 1e-4
        assert rel(gx2s[i].cpu(), gxs[i].cpu()) < 1e-4
        assert rel(gf2s[i].cpu(), gfs[i].cpu()) < 1e-4
        assert rel(l2s[i].cpu(), losses[i].cpu()) < 1e-4
    for i, (plan, x, f, y_obs) in enumerate(cls):
        y1 = plan.forward_both(x, f)
        assert rel(ys[i].cpu(), y1.cpu()) < 1e-6
        l1, gx1, gf1 = plan.loss_grad(x, f, y_obs)
        assert rel(gxs[i].cpu(), gx1.cpu()) < TOL
        assert rel(gfs[i].cpu(), gf1.cpu()) < TOL
        assert rel(losses[i].cpu(), l1.cpu()) < 1e-6


def test_persistent_batch_matches_oracle(cuda):
    from vmbd_gb300.eff import EffBatch
    cls = [make_class(s, c, cuda, 7 * i) for i, (s, c) in enumerate(zip(SMALL, (1, 2, 1)))]
    B = EffBatch([c[0] for c in cls], (1, 2, 1))
    ys = B.forward_both([c[1] for c in cls], [c[2] for c in cls])
    for i, (plan, x, f, _) in enumerate(cls):
        wa = plan.winaux
        g = eff64.Geometry(wa.sx, plan.sf, wa.csf, wa.sw, wa.nhop, "valid")
        for b in range(x.shape[0]):
            ref = eff64.forward(x[b].cpu().numpy(), f[b].cpu().numpy(), g, wa.ws.astype(np.float64))
            assert rel(ys[i][b].cpu(), ref) < TOL


def test_autotuner_picks_a_strategy(cuda):
    from vmbd_gb300 import autotune
    cls = [make_class(s, c, cuda, 3 * i) for i, (s, c) in enumerate(zip(SMALL, (2, 2, 2)))]
    plans = [c[0] for c in cls]
    args = ([c[1] for c in cls], [c[2] for c in cls], [c[3] for c in cls])
    best, times = autotune.tune(plans, (2, 2, 2), *args)
    cands = autotune.candidates(plans)
    assert best in cands and autotune.parse(best)[0] in autotune.STRATEGIES
    assert all(times[s] > 0 for s in ("persistent", "per_class/cta", "per_class/cluster"))
    ms, _, (losses, gxs, gfs) = autotune.time_step(autotune.BatchRunner(plans, (2, 2, 2), best), *args)
    for i, (plan, x, f, y_obs) in enumerate(cls):
        _, gx1, gf1 = plan.loss_grad(x, f, y_obs)
        assert rel(gxs[i].cpu(), gx1.cpu()) < TOL
        assert rel(gfs[i].cpu(), gf1.cpu()) < TOL


@pytest.mark.parametrize("cand", ["per_class/cta@f192", "per_class/cluster@f192/t256", "persistent@f192"])
def test_frame192_candidates_match_default_frames(cuda, cand):
    """The autotuner's 192-frame candidates give the default frames' results
    (the 384x512 class has extent 139, so it moves from 256 to 192).  The
    observation is half the model image, so the residual is of the model's
    size: a noise-sized residual would amplify the two frames' different
    forward rounding ~100x into the gradients."""
    from vmbd_gb300 import autotune
    cls = [make_class(s, c, cuda, 5 * i) for i, (s, c) in enumerate(zip(WORKLOAD, (1, 2, 1)))]
    cls = [(p, x, f, 0.5 * p.forward_both(x, f)) for p, x, f, _ in cls]
    plans = [c[0] for c in cls]
    assert cand in autotune.candidates(plans)
    runner = autotune.BatchRunner(plans, (1, 2, 1), cand)
    assert sorted(p.N for p in runner.plans) != sorted(p.N for p in plans)
    assert 192 in [p.N for p in runner.plans]
    args = ([c[1] for c in cls], [c[2] for c in cls], [c[3] for c in cls])
    _, _, (losses, gxs, gfs) = autotune.time_step(runner, *args, reps=1, warmup=0)
    for i, (plan, x, f, y_obs) in enumerate(cls):
        l1, gx1, gf1 = plan.loss_grad(x, f, y_obs)
        assert rel(gxs[i].cpu(), gx1.cpu()) < TOL
        assert rel(gfs[i].cpu(), gf1.cpu()) < TOL
        assert rel(losses[i].cpu(), l1.cpu()) < 1e-6
