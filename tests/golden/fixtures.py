"""Load the golden fixtures of this directory.

Small cases store their inputs (x, f, r), the reference's window stack (ws)
and outputs.  The workload-size cases (``LARGE_CASES`` in make_golden.py)
store only the outputs, the seed and PSF kind, and checksums of the inputs:
the inputs are regenerated here from the seeds with the same generators and
checked against the checksums, and the window stack is the host geometry's
(the reference's own stack produced the stored outputs, so a different stack
would show up as a parity failure).
"""
from __future__ import annotations

import glob
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def paths(prefix="ref_"):
    return sorted(glob.glob(os.path.join(HERE, prefix + "*.npz")))


def operator_paths():
    return [p for p in paths() if not os.path.basename(p).startswith("ref_deconv_")]


def deconv_paths():
    return paths("ref_deconv_")


def _sums(a):
    return np.array([np.sum(a, dtype=np.float64), np.sum(np.square(a, dtype=np.float64))])


def load(path):
    from vmbd_gb300 import geometry, synth

    z = np.load(path)
    d = {k: z[k] for k in z.files}
    d["mode"] = str(d["mode"])
    d["name"] = os.path.basename(path)[4:-4]
    if "x" not in d:
        sx, sf, csf = tuple(d["sx"]), tuple(d["sf"]), tuple(d["csf"])
        seed, kind = int(d["seed"]), str(d["kind"])
        K = int(np.prod(csf))
        x = synth.blob_edge_image(sx, seed=seed)
        gen = synth.gaussian_psfs if kind == "gauss" else synth.motion_psfs
        f = gen(K, sf, seed=seed + 100)
        r = np.random.default_rng(seed + 200).standard_normal(d["y"].shape).astype(np.float32)
        for name, a in (("x", x), ("f", f), ("r", r)):
            if not np.allclose(_sums(a), d[name + "_sum"], rtol=1e-12, atol=0):
                raise AssertionError(f"{d['name']}: regenerated {name} differs from the fixture's input")
        wa = geometry.Winaux(sx, csf, tuple(d["sw"]), tuple(d["hop"]))
        d.update(x=x, f=f, r=r, ws=np.asarray(wa.ws, np.float32))
    return d
