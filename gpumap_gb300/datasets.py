"""Seeded synthetic workloads with the shapes and distributions of the
benchmark configurations (the image datasets the reference's loaders expect
are not available, so these stand in for them).
"""
from __future__ import annotations

import numpy as np


def gaussian_mixture(n: int, d: int, n_centers: int = 10, center_scale: float = 4.0,
                     sigma: float = 1.0, seed: int = 0):
    """Isotropic mixture: centres ~ N(0, center_scale^2), within-cluster N(0, sigma^2), equal weights."""
    rng = np.random.default_rng(seed)
    centers = rng.normal(0.0, center_scale, size=(n_centers, d))
    z = rng.integers(0, n_centers, size=n)
    x = centers[z] + rng.normal(0.0, sigma, size=(n, d))
    return x.astype(np.float32), z.astype(np.int32)


def image_like(n: int = 70_000, d: int = 784, n_centers: int = 10, seed: int = 0):
    """Sparse nonnegative centres (Bernoulli(0.2) mask, U(0,1) values) plus
    N(0, 0.1^2) noise, clipped to [0, 1]; equal weights."""
    rng = np.random.default_rng(seed)
    mask = rng.random((n_centers, d)) < 0.2
    centers = np.where(mask, rng.random((n_centers, d)), 0.0).astype(np.float32)
    z = rng.integers(0, n_centers, size=n)
    x = np.empty((n, d), dtype=np.float32)
    step = 8192
    for s in range(0, n, step):
        e = min(n, s + step)
        blk = centers[z[s:e]] + rng.normal(0.0, 0.1, size=(e - s, d)).astype(np.float32)
        np.clip(blk, 0.0, 1.0, out=blk)
        x[s:e] = blk
    return x, z.astype(np.int32)


def cosine_zipf(n: int = 1_000_000, d: int = 128, n_centers: int = 100, s: float = 1.1,
                angular_sigma: float = 0.15, seed: int = 0):
    """Centres uniform on the unit sphere, cluster weights ~ j^-s, angular
    noise sigma (per-coordinate N(0, sigma^2/d)), rows L2-normalised."""
    rng = np.random.default_rng(seed)
    c = rng.normal(size=(n_centers, d))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    w = np.arange(1, n_centers + 1, dtype=np.float64) ** (-s)
    w /= w.sum()
    z = rng.choice(n_centers, size=n, p=w)
    x = np.empty((n, d), dtype=np.float32)
    step = 65536
    for s0 in range(0, n, step):
        e = min(n, s0 + step)
        blk = c[z[s0:e]] + rng.normal(0.0, angular_sigma / np.sqrt(d), size=(e - s0, d))
        blk /= np.linalg.norm(blk, axis=1, keepdims=True)
        x[s0:e] = blk.astype(np.float32)
    return x, z.astype(np.int32)


def mixture_stream(n: int, d: int, n_centers: int, seed: int, chunk: int = 8192):
    """Rows of a seeded isotropic Gaussian mixture (centres ~ N(0, 4^2),
    within-cluster sigma 1, equal weights), generated chunk by chunk in row
    order, so that any prefix of the dataset is the same however it is cut."""
    rng = np.random.default_rng(seed)
    centers = rng.normal(0.0, 4.0, size=(n_centers, d)).astype(np.float32)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        z = rng.integers(0, n_centers, size=m)
        yield (centers[z] + rng.normal(0.0, 1.0, size=(m, d)).astype(np.float32)).astype(np.float32)


def session_specs(count: int, n_lo: int, n_hi: int, dims, seed: int = 0):
    """``count`` dataset descriptions as in the batched and served workloads:
    sizes log-uniform in [n_lo, n_hi], a dimensionality drawn from ``dims``
    (a list of choices, or a (lo, hi) range), 5-20 mixture components; the
    data of dataset i uses seed i."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        if isinstance(dims, tuple):
            d = int(rng.integers(dims[0], dims[1] + 1))
        else:
            d = int(rng.choice(dims))
        out.append({"index": i, "n": n, "d": d, "centers": int(rng.integers(5, 21)), "seed": i})
    return out


def poisson_trace(specs, rate: float, duration: float, rows_lo: int, rows_hi: int, seed: int = 0):
    """Insertion requests arriving as a Poisson process of ``rate`` per
    second for ``duration`` seconds, each for a uniformly chosen dataset
    (among those with rows left) and of a uniform size in [rows_lo, rows_hi];
    returns [(arrival_s, dataset index, rows)].  Requests never exceed a
    dataset's size."""
    rng = np.random.default_rng(seed)
    left = [s["n"] for s in specs]
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        alive = [i for i, v in enumerate(left) if v > 0]
        if not alive:
            break
        i = int(rng.choice(alive))
        r = min(int(rng.integers(rows_lo, rows_hi + 1)), left[i])
        left[i] -= r
        out.append((t, i, r))
    return out
