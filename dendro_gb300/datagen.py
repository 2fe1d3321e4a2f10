"""Seeded synthetic point clouds for the benchmark workloads.

The reference's own point files are not part of its source tree, so the
workloads are regenerated from their stated distributions with numpy's PCG64
generator and a fixed seed per workload:

* ``gaussian``   : per axis N(mean, sigma^2), points outside [0,1)^3 redrawn
* ``lognormal``  : per axis u = exp(N(0,1)), mapped by u / (1 + u) into (0,1)
* ``mixture``    : 1-8 isotropic Gaussians, centres U[0.1,0.9]^3, sigma
                   log-uniform in [0.01, 0.2], equal weights, clipped to
                   [0,1)^3 by redrawing
Points are returned as (n, 3) float64 arrays (x, y, z per row).
"""
from __future__ import annotations

import numpy as np


def _inside(p: np.ndarray) -> np.ndarray:
    return np.all((p >= 0.0) & (p < 1.0), axis=1)


def gaussian(n: int, mean: float = 0.5, sigma: float = 0.1, seed: int = 0) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.empty((n, 3))
    k = 0
    while k < n:
        m = max(1024, int((n - k) * 1.05))
        p = rng.normal(mean, sigma, size=(m, 3))
        p = p[_inside(p)][: n - k]
        out[k : k + len(p)] = p
        k += len(p)
    return out


def lognormal(n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    u = np.exp(rng.standard_normal(size=(n, 3)))
    p = u / (1.0 + u)
    # u/(1+u) < 1 always in exact arithmetic; guard the rounding to 1.0
    np.minimum(p, np.nextafter(1.0, 0.0), out=p)
    return p


def mixture(n: int, rng: np.random.Generator) -> np.ndarray:
    k = int(rng.integers(1, 9))
    centres = rng.uniform(0.1, 0.9, size=(k, 3))
    sig = np.exp(rng.uniform(np.log(0.01), np.log(0.2), size=k))
    out = np.empty((n, 3))
    got = 0
    while got < n:
        m = max(1024, int((n - got) * 1.2))
        comp = rng.integers(0, k, size=m)
        p = centres[comp] + rng.standard_normal(size=(m, 3)) * sig[comp, None]
        p = p[_inside(p)][: n - got]
        out[got : got + len(p)] = p
        got += len(p)
    return out


def cloud_sizes(count: int, lo: float, hi: float, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), size=count))).astype(np.int64)


def workload(name: str, n: int | None = None) -> np.ndarray:
    """Named single-cloud workloads with their default sizes and seeds."""
    if name == "gauss1m":  # plain method, small: 1e6 N(0.5, 0.1^2), seed 0
        return gaussian(n or 1_000_000, 0.5, 0.1, seed=0)
    if name == "lognormal64m":  # scale: 64e6 log-normal, seed 0
        return lognormal(n or 64_000_000, seed=0)
    if name == "gauss16m":  # precision workload: 16e6 N(0.5, 0.15^2), seed 3
        return gaussian(n or 16_000_000, 0.5, 0.15, seed=3)
    raise KeyError(name)


def bumps(xyz_u32: np.ndarray, max_depth: int = 30, seed: int = 3) -> np.ndarray:
    """Right-hand side field of the Poisson workload at node coordinates
    (integers at maxDepth scale): f = sum of 4 Gaussian bumps
    a_i exp(-|x - c_i|^2 / (2 s_i^2)), a ~ U[0.5, 2], c ~ U[0.2, 0.8]^3,
    s ~ U[0.05, 0.15] (seeded)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.uniform(0.5, 2.0, 4)
    c = rng.uniform(0.2, 0.8, (4, 3))
    s = rng.uniform(0.05, 0.15, 4)
    if hasattr(xyz_u32, "is_cuda"):  # node coordinates on the device: FP64 field there
        import torch

        x = (xyz_u32.to(torch.int64) & 0xFFFFFFFF).to(torch.float64) / float(1 << max_depth)
        f = torch.zeros(x.shape[0], dtype=torch.float64, device=x.device)
        for i in range(4):
            ci = torch.tensor(c[i], dtype=torch.float64, device=x.device)
            f += float(a[i]) * torch.exp(-((x - ci) ** 2).sum(1) / (2 * float(s[i]) ** 2))
        return f
    x = np.asarray(xyz_u32, np.float64) / float(1 << max_depth)
    f = np.zeros(len(x))
    for i in range(4):
        f += a[i] * np.exp(-((x - c[i]) ** 2).sum(1) / (2 * s[i] ** 2))
    return f
