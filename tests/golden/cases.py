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


def mat_points():
    return datagen.gaussian(150, 0.5, 0.12, seed=34)


def nodal_function(xyz_u32: np.ndarray) -> np.ndarray:
    """Smooth nodal field used for the matVec fixture (coordinates at maxDepth 30)."""
    c = np.asarray(xyz_u32, np.float64) / float(1 << 30)
    return np.sin(3.0 * c[:, 0]) * np.cos(2.0 * c[:, 1]) + c[:, 2] ** 2 - 0.5


def hashed_nodal_values(xyz_u32: np.ndarray) -> np.ndarray:
    """Rough nodal values in [-0.5, 0.5) from a hash of the node coordinates,
    so that every transfer weight shows in the result (transfer fixtures)."""
    x, y, z = (np.asarray(xyz_u32)[:, i].astype(np.uint64) for i in range(3))
    h = (x * np.uint64(73856093)) ^ (y * np.uint64(19349663)) ^ (z * np.uint64(83492791))
    return (h % np.uint64(1 << 20)).astype(np.float64) / float(1 << 20) - 0.5


def element_factors(octs: np.ndarray) -> np.ndarray:
    """Per-octant (Laplacian, mass) factors in [0.5, 1.5) x [0.25, 2.25) from
    a hash of the octant's anchor and level (Jacobian2 fixtures)."""
    o = np.asarray(octs)
    x, y, z, l = (o[:, i].astype(np.uint64) for i in range(4))
    h = (x * np.uint64(73856093)) ^ (y * np.uint64(19349663)) ^ (z * np.uint64(83492791)) ^ (l * np.uint64(2654435761))
    lap = 0.5 + (h % np.uint64(1024)).astype(np.float64) / 1024.0
    mass = 0.25 + ((h >> np.uint64(10)) % np.uint64(1024)).astype(np.float64) / 512.0
    return np.stack([lap, mass], 1)


def csr_summary(node_xyz: np.ndarray, rows: np.ndarray, cols: np.ndarray, vals: np.ndarray) -> dict:
    """Size-independent summary of an assembled matrix given by entries
    between node indices (duplicates summed): with the nodes in lexicographic
    order of their coordinates, the entry count, a SHA-256 of the sorted
    (row, column) pattern, A v for v = hashed_nodal_values, A 1 and the
    diagonal (assembled-matrix fixtures)."""
    order = np.lexsort(np.asarray(node_xyz).T[::-1])
    rank = np.empty(len(order), np.int64)
    rank[order] = np.arange(len(order))
    r, c = rank[np.asarray(rows, np.int64)], rank[np.asarray(cols, np.int64)]
    key = r * len(order) + c
    u, inv = np.unique(key, return_inverse=True)
    v = np.zeros(len(u))
    np.add.at(v, inv, np.asarray(vals, np.float64))
    ur, uc = u // len(order), u % len(order)
    x = hashed_nodal_values(np.asarray(node_xyz)[order])
    av, a1, dg = (np.zeros(len(order)) for _ in range(3))
    np.add.at(av, ur, v * x[uc])
    np.add.at(a1, ur, v)
    np.add.at(dg, ur[ur == uc], v[ur == uc])
    return {"nnz": np.int64(len(u)), "pattern": sha256_records(np.stack([ur, uc], 1)), "av": av, "a1": a1, "diag": dg}


# assembled-matrix fixtures: name -> points
ASSEMBLE = {
    "gauss400": lambda: datagen.gaussian(400, 0.5, 0.15, seed=38),
    "boundary300": lambda: boundary(300, 39),
}


# transfer fixtures: name -> (points, coarsenings before the fine level)
TRANSFER = {
    "gauss1500": (lambda: datagen.gaussian(1500, 0.5, 0.15, seed=35), 0),
    "gauss1500_l1": (lambda: datagen.gaussian(1500, 0.5, 0.15, seed=35), 1),
    "mixture1500": (lambda: datagen.mixture(1500, np.random.Generator(np.random.PCG64(36))), 0),
    "boundary800": (lambda: boundary(800, 37), 0),
}


def sparse_octants(rng, D: int, lmax: int, keep: float = 0.3, p_split: float = 0.6, n_anc: int = 0,
                   n_dup: int = 0) -> np.ndarray:
    """Octants {x, y, z, level} at maxDepth D for completeOctree: the leaves
    of a random refinement of the root (levels <= lmax), a random subset of
    them (so the set has gaps), plus n_anc ancestors of chosen leaves and
    n_dup repeated octants, shuffled."""
    leaves, stack = [], [(0, 0, 0, 0)]
    while stack:
        x, y, z, lev = stack.pop()
        if lev < lmax and (lev == 0 or rng.random() < p_split):
            h = 1 << (D - lev - 1)
            for c in range(8):
                stack.append((x + (c & 1) * h, y + ((c >> 1) & 1) * h, z + ((c >> 2) & 1) * h, lev + 1))
        else:
            leaves.append((x, y, z, lev))
    octs = np.array(leaves, np.uint32).reshape(-1, 4)
    octs = octs[rng.random(len(octs)) < keep]
    if len(octs) == 0:
        octs = np.array(leaves[:1], np.uint32)
    extra = []
    for _ in range(n_anc):
        x, y, z, lev = octs[rng.integers(len(octs))].tolist()
        if lev >= 2:
            la = int(rng.integers(1, lev))
            m = ~((1 << (D - la)) - 1) & 0xFFFFFFFF
            extra.append((x & m, y & m, z & m, la))
    if extra:
        octs = np.concatenate([octs, np.array(extra, np.uint32)])
    if n_dup:
        octs = np.concatenate([octs, octs[rng.integers(0, len(octs), n_dup)]])
    rng.shuffle(octs)
    return np.ascontiguousarray(octs, np.uint32)


def morton_sort(octs: np.ndarray, D: int) -> np.ndarray:
    """Unique octants in the reference's Morton order (ancestor first)."""
    def key(o):
        x, y, z, lev = (int(v) for v in o)
        m = 0
        for b in range(D):
            m |= (((x >> b) & 1) << (3 * b)) | (((y >> b) & 1) << (3 * b + 1)) | (((z >> b) & 1) << (3 * b + 2))
        return (m << 5) | lev
    uniq = {tuple(int(v) for v in o): o for o in octs}
    return np.array(sorted(uniq.keys(), key=key), np.uint32).reshape(-1, 4)


def complete_inputs():
    """(name, octants, maxDepth, isUnique, isSorted) cases for completeOctree;
    the declared flags are always true of the input."""
    rng = np.random.Generator(np.random.PCG64(2024))
    out = [
        ("empty", np.zeros((0, 4), np.uint32), 8, 0, 0),
        ("root", np.array([[0, 0, 0, 0]], np.uint32), 8, 0, 0),
        ("one_D4", np.array([[4, 8, 0, 2]], np.uint32), 4, 0, 0),
        ("min_corner_D5", np.array([[0, 0, 0, 5]], np.uint32), 5, 1, 1),
        ("max_corner_D5", np.array([[31, 31, 31, 5]], np.uint32), 5, 1, 1),
        ("both_corners_D30", np.array([[0, 0, 0, 30], [2 ** 30 - 1] * 3 + [30]], np.uint32), 30, 1, 1),
    ]
    for i in range(24):
        D = int(rng.choice([3, 6, 10, 20, 30]))
        octs = sparse_octants(rng, D, min(D, int(rng.integers(2, 6))), keep=float(rng.uniform(0.05, 0.8)),
                              n_anc=int(rng.integers(0, 3)), n_dup=int(rng.integers(0, 20)))
        srt = morton_sort(octs, D)
        shuf = srt.copy()
        rng.shuffle(shuf)
        out.append((f"sparse{i}_any", octs, D, 0, 0))
        out.append((f"sparse{i}_sorted", srt, D, 1, 1))
        out.append((f"sparse{i}_unique", shuf, D, 1, 0))
    return out


def morton_rank_order(xyz_u32: np.ndarray, bits: int = 31) -> np.ndarray:
    """Indices that sort points (x, y, z integer coordinates below 2^bits) by
    their Morton key (z above y above x at every bit)."""
    xyz = np.asarray(xyz_u32, np.uint64)
    lo = np.zeros(len(xyz), np.uint64)
    hi = np.zeros(len(xyz), np.uint64)
    for b in range(bits):
        for a in range(3):
            bit = (xyz[:, a] >> np.uint64(b)) & np.uint64(1)
            pos = 3 * b + a
            if pos < 63:
                lo |= bit << np.uint64(pos)
            else:
                hi |= bit << np.uint64(pos - 63)
    return np.lexsort((lo, hi))


def config1_vector(node_xyz: np.ndarray, seed: int = 1, order: np.ndarray | None = None) -> np.ndarray:
    """The plain workload's nodal input vector: uniform in [-1, 1] from
    PCG64(seed), assigned to the nodes in the Morton order of their
    coordinates (so it does not depend on a node numbering).  ``order``:
    morton_rank_order(node_xyz), when already known."""
    if order is None:
        order = morton_rank_order(node_xyz)
    v = np.random.Generator(np.random.PCG64(seed)).uniform(-1.0, 1.0, len(node_xyz))
    out = np.empty(len(node_xyz))
    out[order] = v
    return out


def projection_weights(node_xyz: np.ndarray, k: int) -> np.ndarray:
    """k weight vectors (k x n), uniform in [-1, 1] from PCG64(100 + j), in the
    same Morton assignment as config1_vector: sum_i w_ji y_i summarises a
    nodal result y independently of the node numbering."""
    order = morton_rank_order(node_xyz)
    return np.stack([config1_vector(node_xyz, 100 + j, order) for j in range(k)])


def sha256_records(a: np.ndarray) -> str:
    import hashlib

    return hashlib.sha256(memoryview(np.ascontiguousarray(a))).hexdigest()
