#!/usr/bin/env python
"""EFF forward + both adjoints throughput on GB300 (one JSON line).

Workload (default ``cfg2``): one 512x512 float32 blob+edge image cut into an
8x8 grid of 96x96 patches at 50% overlap (hop 48), 128x128 FFT frame, one
31x31 random-walk motion PSF per patch; ``y_obs = EFF(x, f) + N(0, 0.01^2)``.
One step is the autograd step of ``0.5*||EFF(x, f) - y_obs||^2``: PSF
spectrum, fused forward (which also leaves the windowed-patch spectrum),
residual, fused adjoint giving both gradients.  Metric: image Mpixel/s of
that step.  Inputs are seeded synthetic data (no dataset is distributed).

``value``: device-resident inputs, the step captured in a CUDA graph, the K
timed steps replayed back to back between two CUDA events; the timed steps
rotate through distinct input sets of over twice the L2 in total, so each
step reads inputs from HBM (``per_step_events``: the sum of each step's own
event interval instead; ``l2_flushed``: the step after a 256 MB write, which
also evicts the kernels' code).
``e2e``: the same step through the public API from pinned host buffers
(rotating through as many distinct host input sets), with the host->device
copy of (x, f, y_obs) and the device->host copy of (gx, gf, loss) of every
image inside the timed region, for a stream of images: two buffer pairs and
copy streams, so that the copies of neighbouring images overlap the step
(``e2e.one_at_a_time``: copy in, step, copy out, then the next image).  The
copies and the step of an image are captured in one CUDA graph (memcpy nodes
and the step's kernels), one replay per image.
``--impl reference``: the FP64 oracle port of the reference algorithm on the
host cores (scipy.fft over all cores), same workload.

Multi-GPU (``torchrun``): every rank runs its own image (replicas, weak
scaling, no collective in the data path); value = images of all ranks / max
rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "cfg2": dict(desc="512x512, 8x8 grid of 96x96 patches (hop 48), 31x31 motion PSFs, frame 128",
                 sx=(512, 512), csf=(8, 8), sf=(31, 31), sw=(96, 96), hop=(48, 48), kind="motion"),
    "cfg2_winaux": dict(desc="512x512, 8x8 grid, win2winaux patches 122x122 (hop 61), 31x31 motion PSFs, frame 256",
                        sx=(512, 512), csf=(8, 8), sf=(31, 31), sw=None, hop=None, kind="motion"),
    "cfg1": dict(desc="256x256, 4x4 grid of 64x64 patches (hop 32), 15x15 Gaussian PSFs, frame 128",
                 sx=(256, 256), csf=(4, 4), sf=(15, 15), sw=(64, 64), hop=(32, 32), kind="gauss"),
    # the large single-image stress case, literal patches and win2winaux's own geometry
    "cfg5": dict(desc="2048x2048, 16x16 grid of 192x192 patches (hop 96), 41x41 motion PSFs, frame 256",
                 sx=(2048, 2048), csf=(16, 16), sf=(41, 41), sw=(192, 192), hop=(96, 96), kind="motion"),
    "cfg5_winaux": dict(desc="2088x2088 (valid output 2048x2048), 16x16 grid, win2winaux patches 246x246 "
                             "(hop 123), 41x41 motion PSFs, frame 512",
                        sx=(2088, 2088), csf=(16, 16), sf=(41, 41), sw=None, hop=None, kind="motion"),
}
FLUSH_BYTES = 256 << 20
# the timed steps rotate through distinct input sets totalling over twice the
# 129 MB L2 (at least 4 sets)
L2_BYTES = 129 << 20
# Online multi-frame blind deconvolution: 512x512 frames, 25x25 motion PSFs
# drifting over the sequence on an 8x8 grid, Poisson (peak 1000) + Gaussian
# (0.005) noise, per frame 10 PG PSF steps (simplex) + 5 multiplicative image
# steps with edgetaper.  Latent image 536x536 (valid mode), win2winaux patches
# 120x120 (hop 60), frame 256.
MFBD = dict(sy=(512, 512), sf=(25, 25), csf=(8, 8), frames=100, n_pg=10, n_mu=5)
# Uneven batch: 64 images in one persistent launch per direction: 24 at
# 256x256 (4x4 grid, 15x15 Gaussian PSFs), 24 at 384x512 (6x8, 21x21 motion),
# 16 at 1024x1024 (12x12, 31x31 motion); win2winaux geometry per class.
CFG4 = [((256, 256), (4, 4), (15, 15), "gauss", 24), ((384, 512), (6, 8), (21, 21), "motion", 24),
        ((1024, 1024), (12, 12), (31, 31), "motion", 16)]


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured", float(d.get("sm_max_mhz", 2070.0))
    return 6800.0, "fallback", 2070.0


def make_inputs(w, seed):
    from vmbd_gb300 import geometry, synth
    wa = geometry.win2winaux(w["sx"], w["csf"], 0.5, sw=w["sw"], nhop=w["hop"])
    x = synth.blob_edge_image(w["sx"], seed=seed)
    gen = synth.motion_psfs if w["kind"] == "motion" else synth.gaussian_psfs
    f = gen(wa.K, w["sf"], seed=seed + 1000)
    return wa, x, f


def algorithmic(w, wa, N):
    """Unique fp32 I/O bytes and reference-algorithm FFT flops per image."""
    sx, sf, K = w["sx"], w["sf"], wa.K
    sy = (sx[0] - sf[0] + 1, sx[1] - sf[1] + 1)
    px, pf, py = sx[0] * sx[1] * 4, K * sf[0] * sf[1] * 4, sy[0] * sy[1] * 4
    fft = 5.0 * N * N * np.log2(N * N)  # one complex 2-D FFT, benchFFT convention
    prod = 6.0 * N * N
    return {
        # forward r = F x - y_obs: reads x, f and y_obs, writes r; 3K FFTs + K products
        "forward": (px + pf + 2 * py, K * (3 * fft + prod)),
        # both adjoints: reads r, x, f, writes gx and gf; 4K FFTs + 2K products
        "adjoint": (py + px + pf + px + pf, K * (4 * fft + 2 * prod)),
    }


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [s.strip() for s in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def run_ours(args, rank, world, dev):
    import torch
    from vmbd_gb300.eff import EffPlan

    w = WORKLOADS[args.workload]
    wa, x_np, f_np = make_inputs(w, seed=rank)
    plan = EffPlan(wa, w["sf"], "valid", device=dev)
    N, K = plan.N, plan.K
    # The step's inputs (x, f, y_obs) and outputs (gx, gf, loss) each live in
    # one device buffer, so that the end-to-end step moves them with one copy
    # each way (views into the buffers are what the C ABI is given).
    nx, nf = int(np.prod(plan.sx)), K * int(np.prod(plan.sf))
    ny = int(np.prod(plan.sy))
    inbuf = torch.empty(nx + nf + ny, device=dev)
    x, f = inbuf[:nx].view(plan.sx), inbuf[nx:nx + nf].view((K,) + plan.sf)
    y_obs = inbuf[nx + nf:].view(plan.sy)
    x.copy_(torch.from_numpy(x_np))
    f.copy_(torch.from_numpy(f_np))
    gen = torch.Generator(device=dev).manual_seed(1234 + rank)
    y_obs.copy_(plan.forward_image(x, plan.psf_spectrum(f)))
    y_obs += 0.01 * torch.randn(y_obs.shape, device=dev, generator=gen)

    # static buffers of the step
    fhat = plan.empty_spectrum()
    xhat = plan.empty_spectrum()
    y = torch.empty(plan.sy, device=dev)
    o_loss = ((nx + nf) * 4 + 7) // 8 * 8
    outbuf = torch.empty(o_loss + 8, dtype=torch.uint8, device=dev)
    gx = outbuf[:nx * 4].view(torch.float32).view(plan.sx)
    gf = outbuf[nx * 4:(nx + nf) * 4].view(torch.float32).view((K,) + plan.sf)
    loss = outbuf[o_loss:].view(torch.float64).view(())

    def step():
        # fused forward (x, f, y_obs -> residual + both spectra) and fused
        # adjoints of the residual with its loss
        plan.loss_grad(x, f, y_obs, loss=loss, gx=gx, gf=gf)

    # A stream of distinct images: POOL input sets (x, f, y_obs) of over twice
    # the L2 in total, one captured step per set, replayed in turn, so that
    # every step reads inputs that are not in L2 (no flush needed).
    POOL = max(4, -(-2 * L2_BYTES // (inbuf.numel() * 4)))
    pool = inbuf.unsqueeze(0).repeat(POOL, 1).contiguous()
    sets = [(p_[:nx].view(plan.sx), p_[nx:nx + nf].view((K,) + plan.sf), p_[nx + nf:].view(plan.sy))
            for p_ in pool]
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(stream):
        for _ in range(3):
            step()
        torch.cuda.synchronize(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            step()
        graphs = []
        for xi, fi, yi in sets:
            gi = torch.cuda.CUDAGraph()
            with torch.cuda.graph(gi, stream=stream):
                plan.loss_grad(xi, fi, yi, loss=loss, gx=gx, gf=gf)
            graphs.append(gi)
        torch.cuda.synchronize(dev)

        def timed_graph(n, flushed=False):
            """Sum of the steps' own event intervals in ms (each interval also
            charges its replay's launch latency; a loop that waits for each
            step's result sees about that)."""
            evs = []
            for k in range(n):
                if flushed:
                    flush.fill_(1.0)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                (graph if flushed else graphs[k % POOL]).replay()
                b.record(stream)
                evs.append((a, b))
            torch.cuda.synchronize(dev)
            return sum(a.elapsed_time(b) for a, b in evs)

        def timed_loop(n):
            """n steps replayed back to back between two events, in ms: the
            throughput of a job over a stream of images (the host only issues
            one replay per step, so it stays ahead of the device)."""
            a0 = torch.cuda.Event(enable_timing=True)
            b0 = torch.cuda.Event(enable_timing=True)
            reps = [graphs[k % POOL].replay for k in range(n)]
            a0.record(stream)
            for r_ in reps:
                r_()
            b0.record(stream)
            torch.cuda.synchronize(dev)
            return a0.elapsed_time(b0)

        timed_loop(max(args.warmup, POOL))  # every set once, so that the timed steps see a steady state
        clocks = Clocks(dev.index if dev.index is not None else 0)
        barrier(world)
        torch.cuda.synchronize(dev)
        clocks.start()
        t_ms = timed_loop(args.steps)
        torch.cuda.synchronize(dev)
        barrier(world)
        clk = clocks.stop()
        t_ms = allreduce_max(t_ms, world, dev)
        t_events = allreduce_max(timed_graph(args.steps), world, dev)

        # Independent images on two compute streams (a second plan, so a
        # second workspace; captured steps over the same rotating input
        # sets): the steps of one stream follow one another as above, the
        # two streams' kernels share the GPU.  Reported beside `value`, which
        # is the one-stream figure (each step after the previous, as in an
        # optimiser's loop).
        two_ms = None
        try:
            plan2 = EffPlan(wa, w["sf"], "valid", device=dev)
            out2 = torch.empty_like(outbuf)
            gx2_ = out2[:nx * 4].view(torch.float32).view(plan.sx)
            gf2_ = out2[nx * 4:(nx + nf) * 4].view(torch.float32).view((K,) + plan.sf)
            loss2_ = out2[o_loss:].view(torch.float64).view(())
            stream2 = torch.cuda.Stream(device=dev)
            graphs2 = []
            with torch.cuda.stream(stream2):
                plan2.loss_grad(*sets[0], loss=loss2_, gx=gx2_, gf=gf2_)
                for xi, fi, yi in sets:
                    gi = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(gi, stream=stream2):
                        plan2.loss_grad(xi, fi, yi, loss=loss2_, gx=gx2_, gf=gf2_)
                    graphs2.append(gi)
            torch.cuda.synchronize(dev)

            def two_streams(n):
                a0 = torch.cuda.Event(enable_timing=True)
                b0 = torch.cuda.Event(enable_timing=True)
                a0.record(stream)
                stream2.wait_event(a0)
                reps = [(graphs if k % 2 == 0 else graphs2)[(k // 2) % POOL].replay for k in range(n)]
                for k, r_ in enumerate(reps):
                    with torch.cuda.stream(stream if k % 2 == 0 else stream2):
                        r_()
                e2_ = torch.cuda.Event()
                e2_.record(stream2)
                stream.wait_event(e2_)
                b0.record(stream)
                torch.cuda.synchronize(dev)
                return a0.elapsed_time(b0)

            two_streams(max(args.warmup, POOL))
            two_ms = allreduce_max(two_streams(2 * args.steps), world, dev) / (2 * args.steps)
        except Exception as e:  # reported, not fatal to the headline line
            two_ms = repr(e)[:200]
        # the same step with the L2 flushed before it (one set): data and the
        # kernels' code are then read from HBM (per-step intervals: the loop
        # also holds the flushes)
        timed_graph(args.warmup, flushed=True)
        t_flushed = timed_graph(args.steps, flushed=True) / args.steps

        # per-kernel durations inside the step: differences of graph-captured
        # prefixes of the step's own sequence, input sets rotated
        kern_ms = kernel_times(plan, sets, y, xhat, fhat, gx, gf, loss, stream, dev,
                               reps=max(5, min(args.steps, 50)))

        # the same step on a deterministic plan (fixed-order gather overlap-add)
        det_ms = None
        try:
            dplan = EffPlan(wa, w["sf"], "valid", device=dev, deterministic=True)
            dstep = lambda: dplan.loss_grad(x, f, y_obs, loss=loss, gx=gx, gf=gf)  # noqa: E731
            for _ in range(3):
                dstep()
            torch.cuda.synchronize(dev)
            dg = torch.cuda.CUDAGraph()
            with torch.cuda.graph(dg, stream=stream):
                dstep()
            torch.cuda.synchronize(dev)
            dt = 0.0
            for i in range(args.warmup + args.steps):
                flush.fill_(1.0)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                dg.replay()
                b.record(stream)
                torch.cuda.synchronize(dev)
                if i >= args.warmup:
                    dt += a.elapsed_time(b)
            det_ms = dt / args.steps
        except Exception as e:  # reported, not fatal to the headline line
            det_ms = repr(e)[:200]

        # unfused per-stage comparator (torch ops + cuFFT), graph-captured
        from vmbd_gb300.unfused import UnfusedEff
        U = UnfusedEff(wa, w["sf"], N=N, device=dev)

        def ustep():
            fh = U.psf_spectrum(f)
            yy, xh = U.forward(x, fh)
            rr = yy - y_obs
            U.adjoint(rr, fh, xh)
            return 0.5 * (rr * rr).sum()

        for _ in range(3):
            ustep()
        torch.cuda.synchronize(dev)
        ug = torch.cuda.CUDAGraph()
        with torch.cuda.graph(ug, stream=stream):
            ustep()
        torch.cuda.synchronize(dev)
        ut = 0.0
        for i in range(args.warmup + args.steps):
            flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ug.replay()
            b.record(stream)
            torch.cuda.synchronize(dev)
            if i >= args.warmup:
                ut += a.elapsed_time(b)
        unfused_ms = ut / args.steps

        # End to end through the public API from pinned host buffers: per
        # image, one host->device copy of its inputs (x, f, y_obs) from a
        # rotating pool of distinct pinned host sets (over twice the L2), the
        # step, one device->host copy of its outputs (gx, gf, loss).  The
        # copies and the step are captured in CUDA graphs (memcpy nodes + the
        # step's kernels), one replay per image, so that the host's speed at
        # issuing calls does not set the number.
        hins = pool.cpu().pin_memory()
        hout = torch.empty(outbuf.shape, dtype=torch.uint8).pin_memory()
        s_in = torch.cuda.Stream(device=dev)
        s_out = torch.cuda.Stream(device=dev)

        # (1) one image at a time: copy in, step, copy out, then the next
        one = []
        for k in range(POOL):
            g1 = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g1, stream=stream):
                inbuf.copy_(hins[k], non_blocking=True)
                step()
                hout.copy_(outbuf, non_blocking=True)
            one.append(g1)
        torch.cuda.synchronize(dev)
        for k in range(args.warmup):
            one[k % POOL].replay()
        torch.cuda.synchronize(dev)
        et_sync = 0.0
        for k in range(args.steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            one[(args.warmup + k) % POOL].replay()
            b.record(stream)
            torch.cuda.synchronize(dev)
            et_sync += a.elapsed_time(b)
        et_sync = allreduce_max(et_sync, world, dev)

        # (2) a stream of images, software-pipelined over two buffer pairs:
        # the replay for image k runs its step on pair k % 2 while, on two
        # other streams inside the same graph, image k+1 is copied into the
        # other pair and image k-1's outputs are copied out of it (each
        # image still makes both copies; the last image's copy-out follows
        # the loop, inside the timed region)
        inbuf2 = torch.empty_like(inbuf)
        outbuf2 = torch.empty_like(outbuf)
        pairs = [(inbuf, outbuf), (inbuf2, outbuf2)]
        houts = [hout, torch.empty_like(hout).pin_memory()]

        def pair_step(i):
            ib, ob = pairs[i]
            plan.loss_grad(ib[:nx].view(plan.sx), ib[nx:nx + nf].view((K,) + plan.sf), ib[nx + nf:].view(plan.sy),
                           loss=ob[o_loss:].view(torch.float64).view(()),
                           gx=ob[:nx * 4].view(torch.float32).view(plan.sx),
                           gf=ob[nx * 4:(nx + nf) * 4].view(torch.float32).view((K,) + plan.sf))

        POOLE = POOL + POOL % 2  # even, so that image k's pair is k % 2 for every replay
        piped = []
        for k in range(POOLE):
            i = k % 2
            gp = torch.cuda.CUDAGraph()
            with torch.cuda.graph(gp, stream=stream):
                s_in.wait_stream(stream)
                s_out.wait_stream(stream)
                with torch.cuda.stream(s_in):
                    pairs[1 - i][0].copy_(hins[(k + 1) % POOL], non_blocking=True)
                with torch.cuda.stream(s_out):
                    houts[1 - i].copy_(pairs[1 - i][1], non_blocking=True)
                pair_step(i)
                stream.wait_stream(s_in)
                stream.wait_stream(s_out)
            piped.append(gp)
        torch.cuda.synchronize(dev)

        def pipelined(n):
            inbuf.copy_(hins[0], non_blocking=True)
            for k in range(n):
                piped[k % POOLE].replay()
            houts[(n - 1) % 2].copy_(pairs[(n - 1) % 2][1], non_blocking=True)

        pipelined(max(args.warmup, 4))
        torch.cuda.synchronize(dev)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        pipelined(args.steps)
        b.record(stream)
        torch.cuda.synchronize(dev)
        et = allreduce_max(a.elapsed_time(b), world, dev)
    h2d = hins[0].numel() * 4
    d2h = hout.numel()
    step()
    plan.forward_both(x, f, out=y, xhat_out=xhat, fhat_out=fhat)
    torch.cuda.synchronize(dev)
    return dict(plan=plan, wa=wa, w=w, x_np=x_np, f_np=f_np, y_obs=y_obs.cpu().numpy(),
                gx=gx.cpu().numpy(), gf=gf.cpu().numpy(), y=y.cpu().numpy(), t_ms=t_ms, t_events=t_events,
                two_ms=two_ms,
                kern_ms=kern_ms, unfused_ms=unfused_ms, e2e_ms=et, e2e_sync_ms=et_sync, h2d=h2d, d2h=d2h, clocks=clk,
                det_ms=det_ms,
                t_flushed=t_flushed, pool=POOL)


def kernel_times(plan, sets, r, xhat, fhat, gx, gf, loss, stream, dev, reps):
    """Device time each kernel adds to the graph-captured step: the step's own
    sequence (the zero kernel clearing the residual, which the fused residual
    forward overlaps; the forward, clearing the adjoint's accumulators as a
    side job; the fused adjoint) captured as prefixes -- clear + forward, the
    whole step -- beside the forward alone (its output taken as already
    cleared: timing only) and a one-node graph (a memset of the residual: the
    launch cost every graph pays), for every input set, replayed in turn
    (inputs not in L2, as for the timed steps) and timed with CUDA events:
    forward = T(forward) - T(one node), clear = T(clear + forward) -
    T(forward), adjoint = T(step) - T(clear + forward).  Each includes its
    launch gap in the graph."""
    import ctypes
    import torch
    from vmbd_gb300 import _lib
    from vmbd_gb300.eff import _ptr
    L = plan.lib
    st = ctypes.c_void_p(stream.cuda_stream)
    nx = int(np.prod(plan.sx))

    def seq(n, x, f, y_obs):
        if n == 0:
            r.zero_()  # a graph of one node: the launch cost the others share
        if n in (1, 2, 3):
            # n = 1, 2: the step's clear of the residual (a zero kernel) and
            # its forward; n = 3: the forward alone
            _lib.check(L.eff_forward_both_ex(plan._h, _ptr(x), _ptr(f), _ptr(y_obs), _ptr(r), _ptr(xhat),
                                             _ptr(fhat), _lib.OUT_ZEROED if n == 3 else 0, _ptr(gx), nx,
                                             _ptr(loss), 1, 1, st))
        if n == 2:
            _lib.check(L.eff_adjoint_ex(plan._h, _ptr(r), None, None, _ptr(fhat), _ptr(xhat), _ptr(gx), _ptr(gf),
                                        _ptr(loss), _lib.ADJ_EXACT,
                                        _lib.OUT_ZEROED | _lib.LOSS_OF_Y | _lib.AFTER_FORWARD, 1, st))

    graphs = [[], [], [], []]
    with torch.cuda.stream(stream):
        for n in range(4):
            seq(n, *sets[0])
            torch.cuda.synchronize(dev)
            for xs in sets:
                gph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(gph, stream=stream):
                    seq(n, *xs)
                graphs[n].append(gph)
        torch.cuda.synchronize(dev)
        tot = [0.0, 0.0, 0.0, 0.0]
        np_ = len(sets)
        for i in range(np_ + reps):
            for n in range(4):  # interleaved, so that all four see the same conditions
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                graphs[n][i % np_].replay()
                b.record(stream)
                torch.cuda.synchronize(dev)
                if i >= np_:
                    tot[n] += a.elapsed_time(b)
    t = [v / reps for v in tot]
    return {"forward": t[3] - t[0], "clear": t[1] - t[3], "adjoint": t[2] - t[1], "graph_one_node": t[0],
            "how": "differences of graph-replayed prefixes of the step (one-node graph | forward alone | "
                   "clear + forward | + adjoint), input sets rotated"}


def profile_run(args, dev):
    """The step, eagerly, warmup + steps times (no graph, no comparators)."""
    import torch
    from vmbd_gb300.eff import EffPlan
    if args.workload == "mfbd":
        from vmbd_gb300.mfbd import OnlineMFBD, make_sequence
        M = OnlineMFBD(MFBD["sy"], MFBD["sf"], MFBD["csf"], n_pg=MFBD["n_pg"], n_mu=MFBD["n_mu"], device=dev)
        _, _, ys = make_sequence(M.plan, args.warmup + args.steps, seed=11)
        M.init_latent(ys[:1])
        for t in range(args.warmup + args.steps):
            M.frame(ys[t])
        torch.cuda.synchronize(dev)
        print(json.dumps({"profile": "mfbd", "frames": args.warmup + args.steps}))
        return
    if args.workload == "deconv":
        # Fourier-division deconvolution on the 512^2 / 8x8 / 96^2 / 31^2 geometry:
        # image and PSF estimates from one call per step
        w = WORKLOADS["cfg2"]
        wa, x_np, f_np = make_inputs(w, seed=3)
        plan = EffPlan(wa, w["sf"], "valid", device=dev)
        x = torch.from_numpy(x_np).to(dev)
        f = torch.from_numpy(f_np).to(dev)
        fh, xh = plan.psf_spectrum(f), plan.image_spectrum(x)
        y = plan.forward_image(x, fh)
        flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
        for _ in range(args.warmup + args.steps):
            flush.fill_(1.0)
            plan.deconv_xdirect(y, fhat=fh, xhat=xh, alpha=1e-2, beta=1e-2)
        torch.cuda.synchronize(dev)
        print(json.dumps({"profile": "deconv", "steps": args.warmup + args.steps}))
        return
    if args.workload == "cfg4":
        # one autotuner candidate (--candidate), eagerly, without the tuning runs
        from vmbd_gb300 import autotune
        plans, counts, xs, fs, yo = cfg4_data(dev)
        runner = autotune.BatchRunner(plans, counts, args.candidate)
        losses = [torch.empty(c, dtype=torch.float64, device=dev) for c in counts]
        gxs = [torch.empty((c,) + p.sx, device=dev) for p, c in zip(plans, counts)]
        gfs = [torch.empty((c, p.K) + p.sf, device=dev) for p, c in zip(plans, counts)]
        for _ in range(args.warmup + args.steps):
            runner.loss_grad(xs, fs, yo, losses, gxs, gfs)
        torch.cuda.synchronize(dev)
        print(json.dumps({"profile": "cfg4", "candidate": args.candidate, "steps": args.warmup + args.steps}))
        return
    w = WORKLOADS[args.workload]
    wa, x_np, f_np = make_inputs(w, seed=0)
    plan = EffPlan(wa, w["sf"], "valid", device=dev)
    x = torch.from_numpy(x_np).to(dev)
    f = torch.from_numpy(f_np).to(dev)
    y_obs = plan.forward_image(x, plan.psf_spectrum(f))
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup + args.steps):
        flush.fill_(1.0)
        plan.loss_grad(x, f, y_obs)
    torch.cuda.synchronize(dev)
    print(json.dumps({"profile": args.workload, "steps": args.steps, "warmup": args.warmup}))


def run_mfbd(args, dev, n_timed, with_unfused=True, with_parity=True):
    """Frames/s of the online MFBD loop, one frame per step, graph-captured."""
    import torch
    from vmbd_gb300.mfbd import OnlineMFBD, make_sequence
    from vmbd_gb300.unfused import UnfusedMFBD
    M = OnlineMFBD(MFBD["sy"], MFBD["sf"], MFBD["csf"], n_pg=MFBD["n_pg"], n_mu=MFBD["n_mu"], device=dev)
    _, _, ys = make_sequence(M.plan, MFBD["frames"], seed=11)
    M.init_latent(ys[:20])
    x0, f0 = M.x.clone(), M.f.clone()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    nf = MFBD["frames"]
    with torch.cuda.stream(stream):
        M.frame(ys[0])
        torch.cuda.synchronize(dev)
        M.x.copy_(x0)
        M.f.copy_(f0)
        gph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gph, stream=stream):
            M.frame(None)
        torch.cuda.synchronize(dev)

        def timed(replay, total):
            t = 0.0
            for i in range(total):
                flush.fill_(1.0)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                replay(i % nf)
                b.record(stream)
                torch.cuda.synchronize(dev)
                if i >= args.warmup:
                    t += a.elapsed_time(b)
            return t / (total - args.warmup)

        def ours(i):
            M.y.copy_(ys[i])
            gph.replay()

        ms = timed(ours, args.warmup + n_timed)
        out = {"value": 1e3 / ms, "unit": "frames/s", "ms_per_frame": ms,
               "config": "512x512 frames, 8x8 grid (win2winaux 120x120 patches, hop 60, frame 256), "
                         "25x25 drifting motion PSFs, Poisson peak 1000 + N(0, 0.005^2); per frame "
                         "edgetaper + 10 PG (simplex) + 5 multiplicative steps",
               "gpu_launches_per_frame": M.launches_per_frame(),
               "psf_sum_dev": float((M.f.sum(dim=(1, 2)) - 1).abs().max())}
        if with_unfused:
            U = UnfusedMFBD(M)
            ux = torch.empty_like(M.x).copy_(x0)
            uf = torch.empty_like(M.f).copy_(f0)
            uy = torch.empty_like(M.y)
            U.frame(ys[0], ux, uf)
            torch.cuda.synchronize(dev)
            ug = torch.cuda.CUDAGraph()
            with torch.cuda.graph(ug, stream=stream):
                nx, nf_ = U.frame(uy, ux, uf)
                ux.copy_(nx)
                uf.copy_(nf_)
            torch.cuda.synchronize(dev)

            def unfused(i):
                uy.copy_(ys[i])
                ug.replay()

            ums = timed(unfused, args.warmup + max(5, n_timed // 4))
            out["unfused_gpu"] = {"value": 1e3 / ums, "ms_per_frame": ums, "speedup": ums / ms}
    if with_parity:
        out["rel_l2_vs_fp64_oracle"] = mfbd_parity(M, ys[0], x0, f0)
    return out


def mfbd_parity(M, y, x0, f0):
    """Relative L2 of one MFBD frame against the FP64 oracle, from the same
    start (x0, f0): per step, every kernel output (PSF gradient, F^T(m y),
    F^T(m F x)) against the oracle applied to the GPU's own state before the
    step (worst over the frame), and the frame's result (PSFs and image after
    10 PG + 5 multiplicative steps) against the oracle's own frame."""
    import torch
    from oracle import eff64, mfbd64
    dev = M.device
    wa = M.winaux
    g = eff64.Geometry(M.sx, M.sf, wa.csf, wa.sw, wa.nhop, "valid")
    ws = wa.ws.astype(np.float64)
    eff64.set_fft_workers(os.cpu_count() or 1)

    def h(t):
        return t.detach().double().cpu().numpy()

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))

    M.x.copy_(x0)
    M.f.copy_(f0)
    M.state.fill_(1.0)
    M.begin_frame(y)
    torch.cuda.synchronize(dev)
    yt = h(M.y)
    mask = (yt < 1).astype(np.float64)
    x = h(M.x)
    worst = {"psf_gradient": 0.0, "image_num": 0.0, "image_den": 0.0}
    for k in range(M.n_pg):
        fk = h(M.f)
        M.psf_step(k)
        torch.cuda.synchronize(dev)
        g64 = eff64.adjoint_psf(eff64.forward(x, fk, g, ws) - yt, x, g, ws)
        worst["psf_gradient"] = max(worst["psf_gradient"], rel(h(M.g), g64))
    f = h(M.f)
    M.begin_image_steps()
    torch.cuda.synchronize(dev)
    worst["image_num"] = rel(h(M.num), eff64.adjoint_image(mask * yt, f, g, ws))
    for i in range(M.n_mu):
        xi = h(M.x)
        M.image_step(i)
        torch.cuda.synchronize(dev)
        den64 = eff64.adjoint_image(mask * eff64.forward(xi, f, g, ws), f, g, ws)
        worst["image_den"] = max(worst["image_den"], rel(h(M.den), den64))
    xo, fo, _, _ = mfbd64.mfbd_frame(h(x0), h(f0), y.double().cpu().numpy(), g, ws, M.n_pg, M.n_mu,
                                     state=1.0)
    eff64.set_fft_workers(None)
    return {"per_step_worst": worst, "frame_psfs": rel(h(M.f), fo), "frame_image": rel(h(M.x), xo),
            "note": "per step: each kernel output vs the oracle applied to the GPU's state before the step; "
                    "frame: PSFs and image after one whole frame vs the oracle's own frame from the same "
                    "start (rounding propagated through 15 dependent steps)"}


def run_deconv(args, dev, n_timed):
    """Fourier-division deconvolution (OlaGPU.deconv 'xdirect') on the 512^2
    8x8 / 96^2-patch / 31^2-PSF geometry (frame 128): one call estimates the
    image (F object) and the PSFs (X object) from one transform of y."""
    import torch
    from vmbd_gb300.eff import EffPlan
    from vmbd_gb300.unfused import UnfusedEff
    w = WORKLOADS["cfg2"]
    wa, x, f = make_inputs(w, seed=3)
    plan = EffPlan(wa, w["sf"], "valid", device=dev)
    U = UnfusedEff(wa, w["sf"], "valid", N=plan.N, device=dev)
    xt = torch.from_numpy(x).to(dev)
    ft = torch.from_numpy(f).to(dev)
    fh, xh = plan.psf_spectrum(ft), plan.image_spectrum(xt)
    y = plan.forward_image(xt, fh)
    y = y + 0.01 * torch.randn(y.shape, device=dev, generator=torch.Generator(device=dev).manual_seed(5))
    ufh, uxh = U.psf_spectrum(ft), U.image_spectrum(xt)
    alpha, beta = 1e-2, 1e-2
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def timed(fn, total):
        t = 0.0
        with torch.cuda.stream(stream):
            for i in range(total):
                flush.fill_(1.0)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                torch.cuda.synchronize(dev)
                if i >= args.warmup:
                    t += a.elapsed_time(b)
        return t / (total - args.warmup)

    ms = timed(lambda: plan.deconv_xdirect(y, fhat=fh, xhat=xh, alpha=alpha, beta=beta), args.warmup + n_timed)
    ums = timed(lambda: U.xdirect(y, ufh, uxh, alpha, beta), args.warmup + n_timed)
    u, fz = plan.deconv_xdirect(y, fhat=fh, xhat=xh, alpha=alpha, beta=beta)
    torch.cuda.synchronize(dev)
    px = w["sx"][0] * w["sx"][1]
    out = {"value": px / (ms * 1e-3) / 1e6, "unit": "Mpixel/s", "ms_per_call": ms,
           "config": w["desc"] + "; image + PSF estimates from one call, alpha 0.01, beta 0.01",
           "unfused_gpu": {"ms_per_call": ums, "speedup": ums / ms}}
    check = dict(wa=wa, sf=w["sf"], N=plan.N, x=x, f=f, y=y.cpu().numpy(), u=u.cpu().numpy(),
                 fz=fz.cpu().numpy(), alpha=alpha, beta=beta)
    return out, check


def deconv_parity(c):
    """Relative L2 of the deconvolution outputs against the FP64 oracle, and
    of the oracle's all-FP32 restatement (the error any FP32 pipeline has)."""
    from oracle import eff64
    wa = c["wa"]
    g = eff64.Geometry(wa.sx, c["sf"], wa.csf, wa.sw, wa.nhop, "valid", (c["N"], c["N"]))
    ws = wa.ws.astype(np.float64)
    a, b, y = c["alpha"], c["beta"], c["y"]
    u_ref = eff64.deconv_xdirect(y, eff64.psf_spectrum(c["f"], g), g, ws, "image", a, b)
    f_ref = eff64.deconv_xdirect(y, eff64.image_spectrum(c["x"], g, ws), g, ws, "psf", a, b)

    def rel(p, q):
        return float(np.linalg.norm(np.asarray(p, np.float64) - q) / np.linalg.norm(q))
    return {"image": rel(c["u"], u_ref), "psf": rel(c["fz"], f_ref),
            "psf_fp32_restatement": rel(eff64.deconv_xdirect_fp32(y, c["x"], g, ws, "psf", a, b), f_ref),
            "note": "PSF estimates divide by |X-hat|^2 (dynamic range ~1e9): an all-FP32 pipeline "
                    "is a few 1e-5 from FP64"}


def cfg4_data(dev):
    """Plans and seeded data of the uneven 64-image batch."""
    import torch
    from vmbd_gb300 import geometry, synth
    from vmbd_gb300.eff import EffPlan
    plans, counts, xs, fs, yo = [], [], [], [], []
    for ci, (sx, csf, sf, kind, count) in enumerate(CFG4):
        wa = geometry.win2winaux(sx, csf, 0.5)
        plan = EffPlan(wa, sf, "valid", device=dev)
        gen = synth.motion_psfs if kind == "motion" else synth.gaussian_psfs
        # 4 distinct seeded images / PSF sets per class, repeated to the count
        xu = np.stack([synth.blob_edge_image(sx, seed=100 * ci + i) for i in range(4)])
        fu = np.stack([gen(wa.K, sf, seed=100 * ci + 50 + i) for i in range(4)])
        x = torch.from_numpy(xu[np.arange(count) % 4]).to(dev)
        f = torch.from_numpy(fu[np.arange(count) % 4]).to(dev)
        y = plan.forward_both(x, f)
        y += 0.01 * torch.randn(y.shape, device=dev, generator=torch.Generator(device=dev).manual_seed(ci))
        plans.append(plan)
        counts.append(count)
        xs.append(x)
        fs.append(f)
        yo.append(y)
    return plans, counts, xs, fs, yo


def run_cfg4(args, dev, n_timed, with_parity=True):
    """Images/s of the loss/gradient step over the uneven 64-image batch with
    the autotuner's strategy (every candidate's time is reported)."""
    from vmbd_gb300 import autotune
    plans, counts, xs, fs, yo = cfg4_data(dev)
    best, times = autotune.tune(plans, counts, xs, fs, yo)
    runner = autotune.BatchRunner(plans, counts, best)
    ms, _, _ = autotune.time_step(runner, xs, fs, yo, reps=max(3, n_timed), warmup=args.warmup)
    n_img = sum(counts)
    items = sum(p.K * c for p, c in zip(plans, counts))
    out = {"value": n_img / (ms * 1e-3), "unit": "images/s", "ms_per_step": ms, "strategy": best,
           "candidates_ms": {k: v for k, v in times.items() if not k.endswith(":error")},
           "patches_per_step": items, "frames": [p.N for p in plans],
           "config": "64 images: 24 x 256^2 (4x4, 15^2 Gaussian), 24 x 384x512 (6x8, 21^2 motion), "
                     "16 x 1024^2 (12x12, 31^2 motion); loss + both gradients per step"}
    if with_parity:
        out["rel_l2_vs_fp64_oracle"] = cfg4_parity(runner.plans, xs, fs, yo)
    return out


def cfg4_parity(plans, xs, fs, yo):
    """Relative L2 against the FP64 oracle on the first image of each class:
    the residual forward and both gradients of the step's two kernels (fused
    residual forward, fused adjoint of that residual) on the plans the chosen
    strategy runs; the adjoints are compared on the same (GPU) residual."""
    import torch
    from oracle import eff64
    eff64.set_fft_workers(os.cpu_count() or 1)

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))

    out = {}
    for p, x, f, y_obs in zip(plans, xs, fs, yo):
        xi, fi, yi = x[0].contiguous(), f[0].contiguous(), y_obs[0].contiguous()
        fh, xh = p.empty_spectrum(), p.empty_spectrum()
        r = p.forward_both(xi, fi, xhat_out=xh, fhat_out=fh, subtract=yi)
        loss, gx, gf = p.adjoint(r, fh, xh, residual=True)
        torch.cuda.synchronize(p.device)
        wa = p.winaux
        g = eff64.Geometry(p.sx, p.sf, wa.csf, wa.sw, wa.nhop, "valid")
        ws = wa.ws.astype(np.float64)
        xn, fn = xi.double().cpu().numpy(), fi.double().cpu().numpy()
        yn = yi.double().cpu().numpy()
        rn = r.double().cpu().numpy()
        y64 = eff64.forward(xn, fn, g, ws)
        out[f"{p.sx[0]}x{p.sx[1]}"] = {
            "forward": rel(rn + yn, y64),
            "adjoint_image": rel(gx.cpu().numpy(), eff64.adjoint_image(rn, fn, g, ws)),
            "adjoint_psf": rel(gf.cpu().numpy(), eff64.adjoint_psf(rn, xn, g, ws)),
            "loss": abs(float(loss) - 0.5 * float(np.sum(rn * rn))) / (0.5 * float(np.sum(rn * rn)))}
    eff64.set_fft_workers(None)
    return out


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(v, world, dev):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def oracle_step(w, wa, x, f, y_obs, r=None):
    """One fwd + both exact adjoints of the FP64 oracle (of residual ``r``
    when given, else of its own ``y - y_obs``)."""
    from oracle import eff64
    g = eff64.Geometry(w["sx"], w["sf"], wa.csf, wa.sw, wa.nhop, "valid")
    ws = wa.ws.astype(np.float64)
    y = eff64.forward(x, f, g, ws)
    if r is None:
        r = y - y_obs
    return y, eff64.adjoint_image(r, f, g, ws), eff64.adjoint_psf(r, x, g, ws)


def cpu_sample(w, wa, x, f, y_obs, r_gpu, budget_s=12.0, max_reps=50, warm=1):
    """Time the oracle step on the host (scipy.fft over all cores); the last
    run's adjoints take the GPU's residual so that they check the kernels."""
    from oracle import eff64
    cores = os.cpu_count() or 1
    eff64.set_fft_workers(cores)
    for _ in range(warm):
        oracle_step(w, wa, x, f, y_obs)
    times, out = [], None
    t_end = time.perf_counter() + budget_s
    while len(times) < max_reps and (not times or time.perf_counter() < t_end):
        t0 = time.perf_counter()
        oracle_step(w, wa, x, f, y_obs)
        times.append(time.perf_counter() - t0)
    out = oracle_step(w, wa, x, f, y_obs, r=r_gpu)
    return statistics.median(times), len(times), cores, out


def cpu_sample_single(w, wa, x, f, y_obs, budget_s=4.0, max_reps=10):
    """The same oracle step with single-threaded numpy.fft (median)."""
    from oracle import eff64
    eff64.set_fft_workers(None)
    times = []
    t_end = time.perf_counter() + budget_s
    while len(times) < max_reps and (not times or time.perf_counter() < t_end):
        t0 = time.perf_counter()
        oracle_step(w, wa, x, f, y_obs)
        times.append(time.perf_counter() - t0)
    return statistics.median(times), len(times)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=list(WORKLOADS) + ["mfbd", "cfg4", "deconv"], default="cfg2")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--candidate", default="persistent",
                    help="uneven-batch strategy for --workload cfg4 --profile (an autotuner candidate)")
    ap.add_argument("--profile", action="store_true",
                    help="short eager run of the step only (for an ncu launch list / capture)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "mfbd" and not args.profile:
        return main_mfbd(args, world, rank, local)
    if args.workload == "cfg4" and not args.profile:
        return main_cfg4(args, world, rank, local)
    if args.workload == "deconv" and not args.profile:
        ap.error("--workload deconv is a --profile mode; its timing is part of the default bench line")
    if args.profile:
        import torch
        torch.cuda.set_device(local)
        profile_run(args, torch.device("cuda", local))
        return
    w = WORKLOADS[args.workload]
    pixels = w["sx"][0] * w["sx"][1]
    metric = "EFF fwd+adjoint Mpixel/s"
    config = {"workload": args.workload, "desc": w["desc"], "step": "loss 0.5||EFF(x, f) - y_obs||^2 and both "
              "gradients: fused residual forward (x, f, y_obs -> r = EFF(x, f) - y_obs, both spectra) + fused "
              "adjoint of r (loss, both gradients)", "images_per_gpu": 1,
              "l2": "inputs larger than L2: the timed steps rotate through distinct input sets of over twice the "
                    "L2 in total", "parallelism": f"replicas x{world}"}
    if w.get("sw") and w.get("hop"):
        cov = [(w["csf"][d] - 1) * w["hop"][d] + w["sw"][d] for d in range(2)]
        if cov != list(w["sx"]):
            config["pixels"] = (f"Mpixel/s counts the whole {w['sx'][0]}x{w['sx'][1]} image; this grid's patches "
                                f"cover {cov[0]}x{cov[1]} of it (the reference arm counts the same way)")

    if args.impl == "reference":
        if rank != 0:
            return
        from vmbd_gb300 import geometry  # noqa: F401
        wa, x, f = make_inputs(w, seed=0)
        from oracle import eff64
        g = eff64.Geometry(w["sx"], w["sf"], wa.csf, wa.sw, wa.nhop, "valid")
        y_obs = eff64.forward(x, f, g, wa.ws.astype(np.float64))
        y_obs = y_obs + 0.01 * np.random.default_rng(1234).standard_normal(y_obs.shape)
        cores = os.cpu_count() or 1
        eff64.set_fft_workers(cores)
        for _ in range(args.warmup):
            oracle_step(w, wa, x, f, y_obs)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            oracle_step(w, wa, x, f, y_obs)
        dt = (time.perf_counter() - t0) / args.steps
        v = pixels / dt / 1e6
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": v, "unit": "Mpixel/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "cpu_baseline": {"value": v, "unit": "Mpixel/s", "cores": cores, "kind": "port",
                             "sample": "one full image per step (FP64 NumPy oracle of the reference "
                                       "algorithm, scipy.fft over all host cores)"},
            "e2e": {"value": v, "unit": "Mpixel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.profile:
        profile_run(args, dev)
        return
    R = run_ours(args, rank, world, dev)
    plan, wa = R["plan"], R["wa"]
    ms = R["t_ms"] / args.steps
    value = world * pixels / (ms * 1e-3) / 1e6
    e2e_ms = R["e2e_ms"] / args.steps
    e2e_sync_ms = R["e2e_sync_ms"] / args.steps
    hbm, hbm_kind, sm_max = peaks()
    alg = algorithmic(w, wa, plan.N)
    kern = {k: v for k, v in R["kern_ms"].items() if k in alg}
    dom = max(kern, key=kern.get)
    bytes_, flops = alg[dom]
    t_dom = kern[dom] * 1e-3
    achieved = bytes_ / t_dom / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", f"traffic_{args.workload}.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp)).get(dom)
    clk = R["clocks"]
    sm_mhz = clk["sm_mhz"] if clk else sm_max
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    line = {
        "metric": metric, "value": value, "unit": "Mpixel/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded blob+edge image, motion PSFs)",
        "config": config,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                     "peak_kind": hbm_kind, "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                     "algorithmic_bytes": bytes_, "kernel_ms": kern[dom],
                     "fp32": {"ref_alg_tflops": flops / t_dom / 1e12, "peak_tflops_at_clock": fp32_peak,
                              "frac": flops / t_dom / 1e12 / fp32_peak},
                     "per_kernel": {k: {"ms": kern[k], "hbm_frac": alg[k][0] / (kern[k] * 1e-3) / 1e9 / hbm,
                                        "fp32_frac": alg[k][1] / (kern[k] * 1e-3) / 1e12 / fp32_peak}
                                    for k in kern}},
        "kernels_ms": R["kern_ms"],
        "unfused_gpu": {"ms_per_step": R["unfused_ms"], "value": world * pixels / (R["unfused_ms"] * 1e-3) / 1e6,
                        "speedup": R["unfused_ms"] / R["t_flushed"],
                        "what": "torch ops + cuFFT per stage, graph-captured; speedup against our step, both "
                                "with the L2 flushed before every step"},
        "e2e": {"value": world * pixels / (e2e_ms * 1e-3) / 1e6, "unit": "Mpixel/s",
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": R["h2d"], "d2h_bytes_per_step": R["d2h"],
                "inputs": f"{R['pool']} distinct pinned host input sets, rotated",
                "how": "a stream of images: each image copied in, processed and copied out, the copies of "
                       "neighbouring images overlapping the step (two buffer pairs, copy streams); copies and "
                       "step captured in one CUDA graph per image, replayed in turn",
                "one_at_a_time": {"value": world * pixels / (e2e_sync_ms * 1e-3) / 1e6, "ms_per_step": e2e_sync_ms,
                                  "how": "copy in, step, copy out (one graph), then the next image"}},
        "two_streams": ({"value": world * pixels / (R["two_ms"] * 1e-3) / 1e6, "ms_per_image": R["two_ms"],
                         "what": "independent images on two compute streams (two plans, the same rotating "
                                 "input sets), graph replays back to back; value is the one-stream figure"}
                        if isinstance(R["two_ms"], float) else {"error": R["two_ms"]}),
        "per_step_events": {"value": world * pixels / (R["t_events"] / args.steps * 1e-3) / 1e6,
                            "ms_per_step": R["t_events"] / args.steps,
                            "what": "the same timed steps, each step's own event interval summed (charges "
                                    "every replay's launch latency; value is the back-to-back loop)"},
        "l2_flushed": {"value": world * pixels / (R["t_flushed"] * 1e-3) / 1e6, "ms_per_step": R["t_flushed"],
                       "what": "the same step with a 256 MB write before it (inputs and the kernels' code "
                               "read from HBM; per-step event intervals)"},
        "input_sets": R["pool"],
        "deterministic": ({"ms_per_step": R["det_ms"], "vs_atomic": R["det_ms"] / R["t_flushed"],
                           "what": "same step on a plan with the fixed-order gather overlap-add (bit-identical "
                                   "repeats): forward + gather + adjoint + gather; L2 flushed before each "
                                   "step, against l2_flushed"}
                          if isinstance(R["det_ms"], float) else {"error": R["det_ms"]}),
        "gpu_launches": 3 * args.steps,  # per step: the residual's clear, the forward, the adjoint
        "clocks": clk,
    }
    if rank == 0 and world == 1:
        try:
            line["mfbd"] = run_mfbd(args, dev, n_timed=20)
        except Exception as e:  # reported, not fatal to the headline line
            line["mfbd"] = {"error": repr(e)[:300]}
        try:
            line["cfg4_batch"] = run_cfg4(args, dev, n_timed=10)
        except Exception as e:
            line["cfg4_batch"] = {"error": repr(e)[:300]}
        deconv_check = None
        try:
            line["deconv_xdirect"], deconv_check = run_deconv(args, dev, n_timed=20)
        except Exception as e:
            line["deconv_xdirect"] = {"error": repr(e)[:300]}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r_gpu = R["y"].astype(np.float64) - R["y_obs"]
        t_cpu, reps, cores, (y_o, gx_o, gf_o) = cpu_sample(w, wa, R["x_np"], R["f_np"], R["y_obs"], r_gpu)
        t1, reps1 = cpu_sample_single(w, wa, R["x_np"], R["f_np"], R["y_obs"])
        line["cpu_baseline"] = {"value": pixels / t_cpu / 1e6, "unit": "Mpixel/s", "cores": cores,
                                "kind": "port",
                                "sample": f"{reps} full-image steps of the same workload (FP64 NumPy "
                                          f"oracle, scipy.fft over {cores} cores), median",
                                "single_thread": {"value": pixels / t1 / 1e6, "cores": 1,
                                                  "sample": f"{reps1} steps, numpy.fft, median"}}

        def rel(a, b):
            return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))
        line["rel_l2_vs_fp64_oracle"] = {"forward": rel(R["y"], y_o), "adjoint_image": rel(R["gx"], gx_o),
                                         "adjoint_psf": rel(R["gf"], gf_o),
                                         "note": "adjoints of the same residual y_gpu - y_obs"}
        if deconv_check is not None:
            line["deconv_xdirect"]["rel_l2_vs_fp64_oracle"] = deconv_parity(deconv_check)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main_cfg4(args, world, rank, local):
    """``--workload cfg4``: images/s of the uneven 64-image batch."""
    import torch
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "metric": "uneven batch images/s",
                              "unavailable": "the reference has no batched path; see --workload cfg2"}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    R = run_cfg4(args, dev, n_timed=args.steps)
    ms = allreduce_max(R["ms_per_step"], world, dev)
    if rank == 0:
        print(json.dumps({
            "metric": "uneven batch images/s", "value": world * 64 / (ms * 1e-3), "unit": "images/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": "cfg4", "desc": R["config"],
                                            "strategy": R["strategy"], "candidates_ms": R["candidates_ms"]},
        }))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main_mfbd(args, world, rank, local):
    """``--workload mfbd``: frames/s of the online MFBD loop as the metric."""
    import torch
    metric = "MFBD frames/s"
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import eff64, mfbd64
        from vmbd_gb300 import geometry, synth
        sy, sf, csf = MFBD["sy"], MFBD["sf"], MFBD["csf"]
        sx = tuple(sy[d] + sf[d] - 1 for d in range(2))
        wa = geometry.win2winaux(sx, csf, 0.5)
        g = eff64.Geometry(sx, sf, wa.csf, wa.sw, wa.nhop, "valid")
        ws = wa.ws.astype(np.float64)
        xt = synth.blob_edge_image(sx, seed=11)
        fs = synth.drifting_motion_psfs(4, wa.K, sf, seed=12)
        cores = os.cpu_count() or 1
        eff64.set_fft_workers(cores)
        rng = np.random.default_rng(13)
        x = np.pad(xt[sf[0] // 2:sf[0] // 2 + sy[0], sf[1] // 2:sf[1] // 2 + sy[1]],
                   ((sf[0] // 2, sf[0] - 1 - sf[0] // 2), (sf[1] // 2, sf[1] - 1 - sf[1] // 2)), mode="edge")
        f = np.full((wa.K,) + sf, 1.0 / (sf[0] * sf[1]))
        state = 1.0
        times = []
        for t in range(args.warmup + args.steps):
            y = eff64.forward(xt, fs[t % 4], g, ws) + 0.005 * rng.standard_normal(g.sy)
            t0 = time.perf_counter()
            x, f, state, _ = mfbd64.mfbd_frame(x, f, y, g, ws, MFBD["n_pg"], MFBD["n_mu"], state=state)
            if t >= args.warmup:
                times.append(time.perf_counter() - t0)
        dt = sum(times) / len(times)
        v = 1.0 / dt
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": v, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "mfbd"},
            "cpu_baseline": {"value": v, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": "one frame per step (FP64 NumPy oracle of the frame loop, "
                                       "scipy.fft over all host cores)"},
            "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    R = run_mfbd(args, dev, n_timed=args.steps)
    ms = allreduce_max(R["ms_per_frame"], world, dev)
    if rank == 0:
        print(json.dumps({
            "metric": metric, "value": world * 1e3 / ms, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "mfbd", "desc": R["config"], "parallelism": f"replicas x{world}",
                       "l2": "flushed (256 MB write) before every timed frame"},
            "unfused_gpu": R.get("unfused_gpu"), "gpu_launches": R["gpu_launches_per_frame"] * args.steps,
        }))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
