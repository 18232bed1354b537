"""Autotuner for batched EFF work: picks the launch strategy, the FFT frame
and the CTA size for a set of geometries by timing the candidates on the
device.

A candidate is ``strategy[@f<frame>][/t<threads>]``:

* strategy ``persistent``: one persistent launch per direction over all
  classes (``EffBatch``; 2-CTA clusters, 512 threads per CTA, one CTA per
  SM -- shared memory is sized for the largest frame of the mix);
  ``per_class/cta``: one batched launch per class and direction, one CTA per
  patch; ``per_class/cluster``: the same with a 2-CTA cluster per patch;
* ``@f192``: classes on the 256 frame whose convolution extent fits run on
  the 192 frame (24 x 8 mixed radix, ~45% less arithmetic, longer per-lane
  chains);
* ``t<n>`` (after ``@``, ``/``-separated from ``f``): CTA size of the
  per-class launches (default: the largest that fits).

Each candidate runs the loss/gradient step (fused forward + fused adjoint),
captured in a CUDA graph, and is timed with CUDA events; the fastest wins.
Results are cached per (geometries, counts, candidates) key for the process.
"""
from __future__ import annotations

import torch

from .eff import EffBatch, EffPlan, set_cluster_mode

_CACHE: dict = {}
STRATEGIES = ("persistent", "per_class/cta", "per_class/cluster")


def _key(plans, counts, cands):
    return tuple((p.sx, p.sf, p.winaux.csf, p.winaux.sw, p.winaux.nhop, p.N, c)
                 for p, c in zip(plans, counts)) + tuple(cands)


def parse(candidate: str):
    """``'per_class/cta@f192/t256'`` -> ('per_class/cta', 192, 256); the
    options after ``@`` are ``f<frame>`` and ``t<threads>``, 0 when absent."""
    strategy, _, tail = candidate.partition("@")
    frame = threads = 0
    for part in tail.split("/") if tail else ():
        if part[:1] == "f" and part[1:].isdigit():
            frame = int(part[1:])
        elif part[:1] == "t" and part[1:].isdigit():
            threads = int(part[1:])
        else:
            raise ValueError(f"bad candidate option {part!r} in {candidate!r}")
    return strategy, frame, threads


def _extent(p):
    return max(p.winaux.sw[d] + p.sf[d] - 1 for d in range(2))


def variant_plans(plans, frame: int = 0, threads: int = 0):
    """The class plans on a smaller frame (the classes whose extent fits it
    and whose own frame is larger; others unchanged) and/or CTA size."""
    out = []
    for p in plans:
        n = frame if frame and _extent(p) <= frame < p.N else p.N
        if n == p.N and not threads:
            out.append(p)
        else:
            out.append(EffPlan(p.winaux, p.sf, p.mode, sfft=n, device=p.device, threads=threads))
    return out


class BatchRunner:
    """The loss/gradient step of a batch with a chosen candidate."""

    def __init__(self, plans, counts, candidate: str):
        strategy, frame, threads = parse(candidate)
        if strategy not in STRATEGIES:
            raise ValueError(f"unknown strategy {strategy!r}")
        self.candidate, self.strategy = candidate, strategy
        self.counts = list(counts)
        self.plans = variant_plans(plans, frame, threads if strategy != "persistent" else 0)
        self.batch = EffBatch(self.plans, counts) if strategy == "persistent" else None

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


def candidates(plans):
    """Every strategy on the power-of-two frames; when a class with extent
    in (128, 192] is not on the 192 frame, every strategy there too, plus the
    per-class strategies with 256-thread CTAs for every class (the 192
    kernels are compiled for up to 384)."""
    out = list(STRATEGIES)
    if any(128 < _extent(p) <= 192 and p.N != 192 for p in plans):
        out += [s + "@f192" for s in STRATEGIES]
        out += [s + "@f192/t256" for s in STRATEGIES if s != "persistent"]
    return tuple(out)


def tune(plans, counts, xs, fs, ys_obs, cands=None):
    """Time every candidate on the given data; returns (best candidate,
    {candidate: ms}).  A candidate that cannot run (shared memory) is
    recorded with its error and skipped."""
    cands = tuple(cands) if cands is not None else candidates(plans)
    key = _key(plans, counts, cands)
    if key in _CACHE:
        return _CACHE[key]
    times = {}
    for c in cands:
        try:
            times[c] = time_step(BatchRunner(plans, counts, c), xs, fs, ys_obs, reps=10, warmup=3)[0]
        except Exception as e:
            times[c] = float("inf")
            times[c + ":error"] = str(e)[:200]
    ran = [c for c in cands if times[c] != float("inf")]
    if not ran:
        errors = {k: v for k, v in times.items() if k.endswith(":error")}
        raise RuntimeError(f"no batch strategy could run on this batch: {errors}")
    best = min(ran, key=lambda c: times[c])
    _CACHE[key] = (best, times)
    return best, times
