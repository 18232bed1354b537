"""Seeded synthetic inputs for the EFF workloads.

The reference measures on a bundled PNG sequence and LSST frames that are not
reproduced here; these generators stand in with images and PSFs of the same
shapes and value ranges.  All draws come from ``numpy.random.default_rng(seed)``
in FP64 and are returned as float32.

* ``blob_edge_image``: a sum of random Gaussian blobs plus random step edges,
  min-max scaled to [0, 1].
* ``gaussian_psfs``: anisotropic Gaussians, sigma in U[0.8, 3], orientation in
  U[0, pi), clipped at 0 and normalised to unit sum.
* ``motion_psfs``: random-walk blur paths of U{10..25} px splatted into the
  PSF box, smoothed by a 1-px Gaussian and normalised (in the spirit of the
  reference's ``imagetools.randomwalk``, imagetools.py:99-132, written fresh).
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage


def blob_edge_image(shape, seed=0, n_blobs: int = 40, n_edges: int = 10) -> np.ndarray:
    rng = np.random.default_rng(seed)
    H, W = int(shape[0]), int(shape[1])
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    img = np.zeros((H, W))
    scale = max(H, W)
    for _ in range(n_blobs):
        cy, cx = rng.uniform(0, H), rng.uniform(0, W)
        s = rng.uniform(0.01, 0.12) * scale
        a = rng.uniform(0.2, 1.0)
        img += a * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * s * s))
    for _ in range(n_edges):
        th = rng.uniform(0, np.pi)
        py, px = rng.uniform(0, H), rng.uniform(0, W)
        h = rng.uniform(-0.6, 0.6)
        img += h * (((xx - px) * np.cos(th) + (yy - py) * np.sin(th)) > 0)
    img -= img.min()
    img /= max(img.max(), 1e-12)
    return img.astype(np.float32)


def gaussian_psfs(K: int, sf, seed=0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    sf = (int(sf[0]), int(sf[1]))
    yy, xx = np.mgrid[0:sf[0], 0:sf[1]].astype(np.float64)
    yy -= (sf[0] - 1) / 2
    xx -= (sf[1] - 1) / 2
    out = np.empty((K,) + sf)
    for k in range(K):
        s1, s2 = rng.uniform(0.8, 3.0, size=2)
        th = rng.uniform(0, np.pi)
        u = xx * np.cos(th) + yy * np.sin(th)
        v = -xx * np.sin(th) + yy * np.cos(th)
        g = np.maximum(np.exp(-(u * u / (2 * s1 * s1) + v * v / (2 * s2 * s2))), 0)
        out[k] = g / g.sum()
    return out.astype(np.float32)


def _walk(rng, length: int, drift=None):
    """Sub-pixel random-walk path with smoothly turning direction."""
    ang = rng.uniform(0, 2 * np.pi) if drift is None else drift
    pts = [np.zeros(2)]
    for _ in range(int(length)):
        ang += rng.normal(0, 0.5)
        pts.append(pts[-1] + np.array([np.sin(ang), np.cos(ang)]))
    return np.array(pts)


def splat_path(pts: np.ndarray, sf) -> np.ndarray:
    """Bilinear splat of a path into an ``sf`` box, centred on its centroid,
    smoothed by a 1-px Gaussian and normalised."""
    sf = (int(sf[0]), int(sf[1]))
    p = pts - pts.mean(axis=0) + np.array([(sf[0] - 1) / 2, (sf[1] - 1) / 2])
    p[:, 0] = np.clip(p[:, 0], 0, sf[0] - 1.001)
    p[:, 1] = np.clip(p[:, 1], 0, sf[1] - 1.001)
    img = np.zeros(sf)
    # densify the path so consecutive samples are < 0.5 px apart
    dense = []
    for a, b in zip(p[:-1], p[1:]):
        n = max(2, int(np.ceil(np.hypot(*(b - a)) * 4)))
        t = np.linspace(0, 1, n, endpoint=False)[:, None]
        dense.append(a + t * (b - a))
    dense.append(p[-1:])
    for y, x in np.concatenate(dense):
        i, j = int(y), int(x)
        fy, fx = y - i, x - j
        img[i, j] += (1 - fy) * (1 - fx)
        img[i + 1, j] += fy * (1 - fx)
        img[i, j + 1] += (1 - fy) * fx
        img[i + 1, j + 1] += fy * fx
    img = ndimage.gaussian_filter(img, 1.0, mode="constant")
    img = np.maximum(img, 0)
    return img / img.sum()


def motion_psfs(K: int, sf, seed=0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.empty((K, int(sf[0]), int(sf[1])))
    for k in range(K):
        L = int(rng.integers(10, 26))
        L = min(L, max(2, min(int(sf[0]), int(sf[1])) - 4))
        out[k] = splat_path(_walk(rng, L), sf)
    return out.astype(np.float32)


def drifting_motion_psfs(n_frames: int, K: int, sf, seed=0) -> np.ndarray:
    """PSF sets for ``n_frames`` frames whose blur paths drift smoothly:
    each patch's path interpolates between two random walks over the frames."""
    rng = np.random.default_rng(seed)
    out = np.empty((n_frames, K, int(sf[0]), int(sf[1])), dtype=np.float32)
    for k in range(K):
        L = int(rng.integers(10, 26))
        L = min(L, max(2, min(int(sf[0]), int(sf[1])) - 4))
        a, b = _walk(rng, L), _walk(rng, L)
        for t in range(n_frames):
            s = 0.5 - 0.5 * np.cos(np.pi * t / max(1, n_frames - 1))
            out[t, k] = splat_path((1 - s) * a + s * b, sf)
    return out
