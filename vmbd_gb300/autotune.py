"""Autotuner for batched EFF work: picks the launch strategy and per-patch
tiling for a set of geometries by timing the candidates on the device.

Candidates for a batch of (plan, count) classes:

* ``persistent``: one persistent launch per direction over all classes
  (``EffBatch``; 2-CTA clusters, 256 threads per CTA);
* ``per_class/cta``: one batched launch per class and direction, one CTA
  per patch (512 threads for frames up to 128, 256 for 256);
* ``per_class/cluster``: the same with a 2-CTA cluster per patch.

Each candidate runs the loss/gradient step (fused forward + fused adjoint),
captured in a CUDA graph, and is timed with CUDA events; the fastest wins.
Results are cached per (geometries, counts) key for the process.
"""
from __future__ import annotations

import torch

from .eff import EffBatch, set_cluster_mode

_CACHE: dict = {}


def _key(plans, counts):
    return tuple((p.sx, p.sf, p.winaux.csf, p.winaux.sw, p.winaux.nhop, p.N, c) for p, c in zip(plans, counts))


class BatchRunner:
    """The loss/gradient step of a batch with a chosen strategy."""

    def __init__(self, plans, counts, strategy: str):
        self.plans, self.counts, self.strategy = list(plans), list(counts), strategy
        self.batch = EffBatch(plans, counts) if strategy == "persistent" else None

    def loss_grad(self, xs, fs, ys_obs, losses, gxs, gfs):
        if self.strategy == "persistent":
            return self.batch.loss_grad(xs, fs, ys_obs, losses, gxs, gfs)
        set_cluster_mode(1 if self.strategy.endswith("cta") else 2)
        try:
            for p, x, f, yo, lo, gx, gf in zip(self.plans, xs, fs, ys_obs, losses, gxs, gfs):
                p.loss_grad(x, f, yo, loss=lo, gx=gx, gf=gf)
        finally:
            set_cluster_mode(0)
        return losses, gxs, gfs


def time_step(runner: BatchRunner, xs, fs, ys_obs, reps=5, warmup=2):
    dev = runner.plans[0].device
    losses = [torch.empty(c, dtype=torch.float64, device=dev) for c in runner.counts]
    gxs = [torch.empty((c,) + p.sx, device=dev) for p, c in zip(runner.plans, runner.counts)]
    gfs = [torch.empty((c, p.K) + p.sf, device=dev) for p, c in zip(runner.plans, runner.counts)]
    stream = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(stream):
        runner.loss_grad(xs, fs, ys_obs, losses, gxs, gfs)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            runner.loss_grad(xs, fs, ys_obs, losses, gxs, gfs)
        torch.cuda.synchronize(dev)
        for _ in range(warmup):
            g.replay()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            g.replay()
        b.record(stream)
        torch.cuda.synchronize(dev)
    return a.elapsed_time(b) / reps, g, (losses, gxs, gfs)


def tune(plans, counts, xs, fs, ys_obs, strategies=("persistent", "per_class/cta", "per_class/cluster")):
    """Time every candidate on the given data; returns (best strategy,
    {strategy: ms})."""
    key = _key(plans, counts)
    if key in _CACHE:
        return _CACHE[key]
    times = {}
    for s in strategies:
        try:
            times[s] = time_step(BatchRunner(plans, counts, s), xs, fs, ys_obs)[0]
        except Exception as e:  # a candidate that does not fit (shared memory) is skipped
            times[s] = float("inf")
            times[s + ":error"] = str(e)[:200]
    best = min((s for s in strategies if times[s] != float("inf")), key=lambda s: times[s])
    _CACHE[key] = (best, times)
    return best, times
