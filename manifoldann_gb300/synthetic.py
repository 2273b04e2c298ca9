"""Seeded synthetic workloads with the shapes and value distributions of the
reference's benchmark datasets (which are not shipped here).  All return
row-major float32 arrays [n][d] (one point per row = the memory of a Julia
d x n matrix).

* ``iid_normal``       -- plain exact kNN: N(0,1) entries (N=10k, Q=1k, d=64).
* ``quantized_mixture``-- 784-d points in [0,1] quantised to k/255 from a
                          10-component Gaussian mixture (stand-in for the
                          fashion-mnist / mnist 60k x 784 sets).
* ``angular_clusters`` -- L2-normalised Gaussian blobs around 100 unit centres
                          in R^256 (stand-in for nytimes-256-angular).
* ``manifold_clouds``  -- Swiss rolls, 2-spheres and tori in R^3, zero-padded
                          to 32-d, rotated and noised (uneven batched graphs).
* ``anisotropic_clusters`` -- 1024 Gaussian clusters with per-dimension sigma
                          log-uniform in [0.05, 0.5], d=128 (stand-in for sift-128).
"""
from __future__ import annotations

import numpy as np


def iid_normal(n: int, d: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal((n, d), dtype=np.float32)


def quantized_mixture(n: int, d: int = 784, seed: int = 0, components: int = 10,
                      sigma: float = 0.15, centre_seed: int = 1234) -> np.ndarray:
    """Mixture shared by every call with the same centre_seed; `seed` draws the points."""
    crng = np.random.default_rng(centre_seed)
    centres = crng.uniform(0.1, 0.9, size=(components, d)).astype(np.float32)
    rng = np.random.default_rng(seed)
    comp = rng.integers(0, components, size=n)
    x = centres[comp] + sigma * rng.standard_normal((n, d), dtype=np.float32)
    np.clip(x, 0.0, 1.0, out=x)
    return (np.rint(x * 255.0) / 255.0).astype(np.float32)


def angular_clusters(n: int, d: int = 256, seed: int = 0, centres: int = 100, sigma: float = 0.3,
                     centre_seed: int = 4321) -> np.ndarray:
    crng = np.random.default_rng(centre_seed)
    c = crng.standard_normal((centres, d))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    rng = np.random.default_rng(seed)
    comp = rng.integers(0, centres, size=n)
    x = c[comp].astype(np.float32) + sigma * rng.standard_normal((n, d), dtype=np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    return x.astype(np.float32)


def _swiss_roll(rng, n):
    t = 1.5 * np.pi * (1 + 2 * rng.random(n))
    h = 21 * rng.random(n)
    return np.stack([t * np.cos(t), h, t * np.sin(t)], axis=1) / 10.0


def _sphere(rng, n):
    v = rng.standard_normal((n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _torus(rng, n, R=1.0, r=0.35):
    # uniform on the surface: accept theta with density ~ (R + r cos theta)
    out = np.empty((0, 3))
    while out.shape[0] < n:
        m = 2 * (n - out.shape[0]) + 16
        th = 2 * np.pi * rng.random(m)
        ph = 2 * np.pi * rng.random(m)
        keep = rng.random(m) < (R + r * np.cos(th)) / (R + r)
        th, ph = th[keep], ph[keep]
        p = np.stack([(R + r * np.cos(th)) * np.cos(ph), (R + r * np.cos(th)) * np.sin(ph),
                      r * np.sin(th)], axis=1)
        out = np.concatenate([out, p])
    return out[:n]


def manifold_clouds(count: int = 64, lo: int = 2000, hi: int = 50000, d: int = 32,
                    noise: float = 0.01, seed: int = 0):
    """List of `count` clouds (row-major [n_i][d] float32), sizes log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)
    q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    clouds = []
    for i, n in enumerate(sizes):
        kind = i % 3
        p3 = (_swiss_roll, _sphere, _torus)[kind](rng, int(n))
        x = np.zeros((int(n), d))
        x[:, :3] = p3
        x = x @ q.T + noise * rng.standard_normal((int(n), d))
        clouds.append(x.astype(np.float32))
    return clouds


def anisotropic_clusters(n: int, d: int = 128, seed: int = 0, clusters: int = 1024,
                         centre_seed: int = 777, chunk: int = 1 << 18) -> np.ndarray:
    crng = np.random.default_rng(centre_seed)
    centres = crng.standard_normal((clusters, d)).astype(np.float32)
    sig = np.exp(crng.uniform(np.log(0.05), np.log(0.5), size=(clusters, d))).astype(np.float32)
    rng = np.random.default_rng(seed)
    comp = rng.integers(0, clusters, size=n)
    out = np.empty((n, d), np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        c = comp[s:e]
        out[s:e] = centres[c] + sig[c] * rng.standard_normal((e - s, d), dtype=np.float32)
    return out
