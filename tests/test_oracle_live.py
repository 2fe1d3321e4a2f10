"""The oracle against the reference binary itself, on fresh seeded inputs
(CPU only; skipped where oracle/_ref has not been built from the
reference's sources, as on machines without them): points2Octree and
balanceOctree bit-exact, completeOctree on inputs the reference completes,
and the Hilbert order of the reference's Hilbert build."""
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
