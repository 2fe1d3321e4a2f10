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

The same seed gives the same points bit for bit on every platform: the
exponentials and logarithms of these generators are evaluated with basic
IEEE operations only (``_exp``, ``_ln``), because numpy's vectorised ``exp``
differs in the last bit between x86 (its own AVX-512 code) and other
platforms (the C library), and one bit can move a point across a level-30
cell boundary.
"""
from __future__ import annotations

import decimal
import math

import numpy as np

_DEC = decimal.Context(prec=50)
# ln 2 to 60 digits (a mathematical constant)
_LN2 = decimal.Decimal("0.693147180559945309417232121458176568075500134360255254120680")


def _split_hi(d: decimal.Decimal) -> float:
    """d rounded to a double whose low 32 mantissa bits are zero, so that
    k * hi is exact for |k| < 2^20."""
    b = np.frombuffer(np.float64(float(d)).tobytes(), np.uint64)[0] & np.uint64(0xFFFFFFFF00000000)
    return float(np.frombuffer(b.tobytes(), np.float64)[0])


_LN2_HI = _split_hi(_LN2)
_LN2_LO = float(_DEC.subtract(_LN2, decimal.Decimal(_LN2_HI)))
_INV_LN2 = float(_DEC.divide(1, _LN2))
_EXP_TAYLOR = [1.0 / math.factorial(k) for k in range(14)]


def _exp(x) -> np.ndarray:
    """exp(x) from + - * and ldexp only (within 2 ulp of the true value):
    x = k ln2 + r with |r| <= ln2 / 2 (Cody-Waite split of ln2), the Taylor
    polynomial of degree 13 in r by Horner's rule (truncation error below
    5e-18 relative), scaled by 2^k."""
    x = np.asarray(x, np.float64)
    k = np.rint(x * _INV_LN2)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.full_like(r, _EXP_TAYLOR[13])
    for c in _EXP_TAYLOR[12::-1]:
        p *= r
        p += c
    return np.ldexp(p, k.astype(np.int32), out=p)


def _ln(v: float) -> float:
    """Natural logarithm of a positive scalar, correctly rounded (decimal
    arithmetic)."""
    return float(_DEC.ln(decimal.Decimal(float(v))))


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
    u = _exp(rng.standard_normal(size=(n, 3)))
    p = u / (1.0 + u)
    # u/(1+u) < 1 always in exact arithmetic; guard the rounding to 1.0
    np.minimum(p, np.nextafter(1.0, 0.0), out=p)
    return p


def mixture(n: int, rng: np.random.Generator) -> np.ndarray:
    k = int(rng.integers(1, 9))
    centres = rng.uniform(0.1, 0.9, size=(k, 3))
    sig = _exp(rng.uniform(_ln(0.01), _ln(0.2), size=k))
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
    return np.round(_exp(rng.uniform(_ln(lo), _ln(hi), size=count))).astype(np.int64)


def batch_clouds(count: int = 256, lo: float = 1e4, hi: float = 4e6, seed: int = 2) -> list:
    """The batching workload: ``count`` Gaussian-mixture clouds with sizes
    log-uniform in [lo, hi] (sizes from ``seed``, then every cloud from one
    generator seeded with ``seed``)."""
    sizes = cloud_sizes(count, lo, hi, seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    return [mixture(int(n), rng) for n in sizes]


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
