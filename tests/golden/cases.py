"""Seeded inputs of the golden fixtures (shared by make_golden.py and tests)."""
from __future__ import annotations

import numpy as np

from dendro_gb300 import datagen


def clustered(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0.2, 0.8, size=(4, 3))
    return c[rng.integers(0, 4, n)] + rng.uniform(0, 2.0 ** -27, size=(n, 3))


def boundary(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    p = rng.uniform(0, 1, size=(n, 3))
    hi = np.nextafter(1.0, 0.0)
    for a in range(3):
        sel = rng.random(n) < 0.3
        p[sel, a] = rng.choice([0.0, hi, 0.5, 2.0 ** -30, 1 - 2.0 ** -30], size=sel.sum())
    return p


def with_duplicates(n, seed):
    base = datagen.gaussian(n, 0.5, 0.1, seed=seed)
    return np.concatenate([base, base[::5], base[::11]])


# name: (generator, maxDepth, maxNumPtsPerOctant)
SMALL = {
    "gauss3k": (lambda: datagen.gaussian(3000, 0.5, 0.1, seed=21), 30, 1),
    "lognormal3k": (lambda: datagen.lognormal(3000, seed=22), 30, 1),
    "mixture2k_m2": (lambda: datagen.mixture(2000, np.random.Generator(np.random.PCG64(23))), 30, 2),
    "clustered1k": (lambda: clustered(1000, 24), 30, 1),
    "boundary1500": (lambda: boundary(1500, 25), 30, 1),
    "duplicates": (lambda: with_duplicates(800, 26), 30, 1),
    "gauss2k_depth12": (lambda: datagen.gaussian(2000, 0.5, 0.2, seed=27), 12, 1),
    "gauss2k_m5": (lambda: datagen.gaussian(2000, 0.5, 0.1, seed=28), 30, 5),
    "two": (lambda: np.array([[0.1, 0.1, 0.1], [0.1 + 2.0 ** -30, 0.1, 0.1]]), 30, 1),
    "one": (lambda: np.array([[0.3, 0.6, 0.9]]), 30, 1),
}

LARGE = {
    "gauss20k": (lambda: datagen.gaussian(20000, 0.5, 0.1, seed=31), 30, 1),
    "lognormal100k": (lambda: datagen.lognormal(100000, seed=32), 30, 1),
}


def da_points():
    return datagen.gaussian(1000, 0.5, 0.1, seed=33)


def nodal_function(xyz_u32: np.ndarray) -> np.ndarray:
    """Smooth nodal field used for the matVec fixture (coordinates at maxDepth 30)."""
    c = np.asarray(xyz_u32, np.float64) / float(1 << 30)
    return np.sin(3.0 * c[:, 0]) * np.cos(2.0 * c[:, 1]) + c[:, 2] ** 2 - 0.5
