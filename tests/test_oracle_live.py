"""The oracle against the reference binary itself, on fresh seeded inputs
(CPU only; skipped where oracle/_ref has not been built from the
reference's sources, as on machines without them): points2Octree and
balanceOctree bit-exact, completeOctree on inputs the reference completes,
the Hilbert order of the reference's Hilbert build, and the multigrid level
operators (transfers, Dirichlet operator and diagonal)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from dendro_gb300 import datagen
from tests.golden import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
DRIVER_H = os.path.join(ROOT, "oracle", "_ref_hilbert", "ref_driver")

pytestmark = pytest.mark.skipif(not os.path.exists(DRIVER), reason="reference driver not built here")


def _run(drv, *args, cwd):
    r = subprocess.run([drv, *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=60)
    return r.returncode == 0


def _write_pts(path, p):
    with open(path, "wb") as f:
        f.write(np.uint64(len(p)).tobytes())
        f.write(np.ascontiguousarray(p, np.float64).tobytes())


def _write_oct(path, o):
    with open(path, "wb") as f:
        f.write(np.uint64(len(o)).tobytes())
        f.write(np.ascontiguousarray(o, np.uint32).tobytes())


def _read_oct(path):
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[:8], np.uint64)[0])
    return np.frombuffer(b[8:], np.uint32).reshape(n, 4).copy()


@pytest.mark.parametrize("seed", [101, 202, 303])
def test_construction_and_balance(oracle, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = datagen.mixture(int(rng.integers(500, 4000)), rng)
    depth = int(rng.choice([10, 20, 30]))
    maxpts = int(rng.integers(1, 4))
    with tempfile.TemporaryDirectory() as tmp:
        pf, of, bf = (os.path.join(tmp, f"c.{e}") for e in ("pts", "oct", "bal"))
        _write_pts(pf, pts)
        assert _run(DRIVER, "p2o", pf, depth, maxpts, of, cwd=tmp)
        lin = _read_oct(of)
        assert np.array_equal(lin, oracle.points_to_octree(pts, depth, maxpts))
        if (lin[:, :3].astype(np.uint64) >> depth).any():
            return  # octants outside the domain: the reference's balance aborts (B7)
        assert _run(DRIVER, "bal", of, depth, 1, 0, bf, cwd=tmp)
        assert np.array_equal(_read_oct(bf), oracle.balance(lin, depth))


def test_complete_fresh_inputs(oracle):
    rng = np.random.Generator(np.random.PCG64(77))
    done = 0
    with tempfile.TemporaryDirectory() as tmp:
        fi, fo = os.path.join(tmp, "in.oct"), os.path.join(tmp, "out.oct")
        for _ in range(12):
            D = int(rng.choice([4, 12, 30]))
            octs = cases.sparse_octants(rng, D, min(D, 5), keep=float(rng.uniform(0.1, 0.7)), n_dup=10)
            _write_oct(fi, octs)
            if not _run(DRIVER, "complete", fi, D, 0, 0, fo, cwd=tmp):
                continue  # the reference aborts on this input (B10)
            assert np.array_equal(_read_oct(fo), oracle.complete(octs, D, 0, 0))
            done += 1
    assert done >= 6


@pytest.mark.skipif(not os.path.exists(DRIVER_H), reason="Hilbert build of the reference not built here")
def test_hilbert_order_fresh_cloud(oracle):
    rng = np.random.Generator(np.random.PCG64(88))
    pts = datagen.gaussian(2500, 0.5, 0.15, seed=88)
    with tempfile.TemporaryDirectory() as tmp:
        pf, of, bf = (os.path.join(tmp, f"h.{e}") for e in ("pts", "oct", "bal"))
        _write_pts(pf, pts)
        assert _run(DRIVER_H, "p2o", pf, 30, 1, of, cwd=tmp)
        assert _run(DRIVER_H, "bal", of, 30, 1, 0, bf, cwd=tmp)
        m = oracle.balance(oracle.points_to_octree(pts, 30, 1), 30)
        assert np.array_equal(_read_oct(bf), oracle.hilbert_sort(m, 30))


def _write_vec(path, xyz, v):
    rec = np.zeros(len(v), dtype=[("c", "<u4", (4,)), ("v", "<f8")])
    rec["c"][:, :3] = xyz
    rec["v"] = v
    with open(path, "wb") as f:
        f.write(np.uint64(len(v)).tobytes())
        f.write(rec.tobytes())


def _read_vec(path):
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[:8], np.uint64)[0])
    rec = np.frombuffer(b[8:], dtype=[("c", "<u4", (4,)), ("v", "<f8")], count=n)
    return rec["c"][:, :3].copy(), rec["v"].copy()


def _same_by_coords(xyz, got, ref_xyz, ref, tol):
    mine, theirs = np.lexsort(xyz.T[::-1]), np.lexsort(ref_xyz.T[::-1])
    assert np.array_equal(xyz[mine], ref_xyz[theirs])
    assert np.abs(got[mine] - ref[theirs]).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("seed", [404, 505, 0])
def test_multigrid_operators_fresh_clouds(oracle, seed):
    """The reference's restrictMatVecType1 / prolongMatVecType1 and
    DirichletJacobianMatMult / DirichletJacobianMatGetDiagonal (driver modes
    transfer and dirichlet) against the oracle's on a fresh mixture cloud,
    and (seed 0) on a 50,000-point log-normal cloud (277k octants, 185k
    nodes)."""
    from types import SimpleNamespace

    from oracle.mg_ref import OracleMG

    rng = np.random.Generator(np.random.PCG64(seed))
    pts = datagen.mixture(int(rng.integers(1500, 5000)), rng) if seed else datagen.lognormal(50_000, seed=41)
    fine = oracle.balance(oracle.points_to_octree(pts, 30, 1), 30)
    coarse = oracle.balance(oracle.coarsen(fine, 30), 30)
    fda, cda = oracle.DA(fine, 30), oracle.DA(coarse, 30)
    vf, vc = rng.standard_normal(fda.n_node), rng.standard_normal(cda.n_node)
    ref_file = os.path.join(os.path.dirname(DRIVER), "REF")  # the source tree the driver was built from
    stencils = os.path.join(open(ref_file).read().strip(), "Stencils") if os.path.exists(ref_file) else ""
    if not os.path.isdir(stencils):
        pytest.skip("reference stencil tables not present")
    with tempfile.TemporaryDirectory() as tmp:
        bf, ff, cf, pre = (os.path.join(tmp, n) for n in ("f.oct", "vf", "vc", "out"))
        _write_oct(bf, fine)
        _write_vec(ff, fda.node_xyz, vf)
        _write_vec(cf, cda.node_xyz, vc)
        assert _run(DRIVER, "transfer", bf, 30, stencils, ff, cf, pre, cwd=tmp)
        assert np.array_equal(_read_oct(pre + ".coarse"), coarse)
        two = SimpleNamespace(pmaps=[fda.prolong_map(coarse, cda)], das=[fda, cda])
        _same_by_coords(cda.node_xyz, OracleMG.restrict(two, 0, vf), *_read_vec(pre + ".r"), 1e-14)
        _same_by_coords(fda.node_xyz, OracleMG.prolong(two, 0, vc), *_read_vec(pre + ".p"), 1e-14)
        assert _run(DRIVER, "dirichlet", bf, 30, stencils, ff, pre, cwd=tmp)
        _same_by_coords(fda.node_xyz, fda.dirichlet_matvec(vf), *_read_vec(pre + ".mv"), 1e-14)
        _same_by_coords(fda.node_xyz, fda.dirichlet_diag(), *_read_vec(pre + ".diag"), 1e-14)
