"""Load the golden fixtures of this directory.

Small cases store their inputs (x, f, r), the reference's window stack (ws)
and outputs.  The workload-size cases (``LARGE_CASES`` in make_golden.py)
store x, f and the outputs; the residual r is regenerated here from the
seed (numpy's default generator gives the same values on every machine) and
checked against the stored checksum, and the window stack is the host
geometry's (the reference's own stack produced the stored outputs, so a
different stack would show up as a parity failure).
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
    from vmbd_gb300 import geometry

    z = np.load(path)
    d = {k: z[k] for k in z.files}
    d["mode"] = str(d["mode"])
    d["name"] = os.path.basename(path)[4:-4]
    if "r_sum" in d:
        r = np.random.default_rng(int(d["seed"]) + 200).standard_normal(d["y"].shape).astype(np.float32)
        if not np.allclose(_sums(r), d["r_sum"], rtol=1e-12, atol=0):
            raise AssertionError(f"{d['name']}: regenerated residual differs from the fixture's")
        wa = geometry.Winaux(tuple(d["sx"]), tuple(d["csf"]), tuple(d["sw"]), tuple(d["hop"]))
        d.update(r=r, ws=np.asarray(wa.ws, np.float32))
    return d
