"""Hilbert-ordered records (dg_ctx_set_order(DG_ORDER_HILBERT), the
reference's default build) on the GPU: construction, balance and
completeOctree outputs against the reference's Hilbert build
(tests/golden/ref_hilbert.npz), sortUniquePoints, batches and uploads of
Hilbert-ordered records against the oracle's Hilbert comparison."""
import os

import numpy as np
import pytest

from dendro_gb300 import (DA, Context, Octree, balanceOctree, completeOctree, datagen, points2Octree,
                          points2OctreeBatch, sortUniquePoints)
from tests.golden import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fnv1a(o):
    h = 1469598103934665603
    for byte in np.ascontiguousarray(o, np.uint32).tobytes():
        h ^= byte
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


@pytest.fixture(scope="module")
def hctx():
    c = Context(0)
    c.set_order("hilbert")
    assert c.order == "hilbert"
    yield c
    c.close()


def _same(got, z, key):
    assert len(got) == int(z[f"{key}_n"]) and fnv1a(got) == int(z[f"{key}_fnv"]), key


def test_points_cases_against_hilbert_build(hctx):
    z = np.load(os.path.join(GOLDEN, "ref_hilbert.npz"))
    ran = 0
    for name, (fn, depth, maxpts) in cases.SMALL.items():
        if not bool(z[f"p2o_{name}/finished"]) or name == "boundary1500":
            continue  # boundary1500: octants outside the domain, no Hilbert position
        lin = points2Octree(fn(), maxDepth=depth, maxNumPtsPerOctant=maxpts, ctx=hctx)
        _same(lin.to_numpy(), z, f"p2o_{name}/lin")
        _same(balanceOctree(lin).to_numpy(), z, f"p2o_{name}/bal")
        ran += 1
    assert ran >= 7


def test_complete_against_hilbert_build(hctx):
    z = np.load(os.path.join(GOLDEN, "ref_hilbert.npz"))
    ran = 0
    for name, octs, D, u, s in cases.complete_inputs():
        key = f"complete_{name}"
        if f"{key}/finished" not in z.files or not bool(z[f"{key}/finished"]):
            continue
        _same(completeOctree(octs, D, ctx=hctx).to_numpy(), z, f"{key}/out")
        ran += 1
    assert ran >= 20


def test_large_and_sort_unique(hctx, ctx, oracle):
    pts = datagen.lognormal(300_000, seed=12)
    m = balanceOctree(points2Octree(pts, ctx=ctx)).to_numpy()
    h = balanceOctree(points2Octree(pts, ctx=hctx)).to_numpy()
    assert np.array_equal(h, oracle.hilbert_sort(m, 30))
    dup = np.concatenate([pts[:50_000], pts[:20_000]])
    assert np.array_equal(sortUniquePoints(dup, ctx=hctx), oracle.hilbert_sort(sortUniquePoints(dup, ctx=ctx), 30))


def test_upload_hilbert_records(hctx, ctx, oracle):
    """Hilbert-ordered records are taken in: a DA on them equals the DA on
    the Morton-ordered records, and they come back out unchanged."""
    pts = datagen.gaussian(20_000, 0.5, 0.1, seed=13)
    m = balanceOctree(points2Octree(pts, ctx=ctx)).to_numpy()
    h = oracle.hilbert_sort(m, 30)
    o = Octree.from_numpy(h, 30, ctx=hctx)
    assert np.array_equal(o.to_numpy(), h)
    da_h, da_m = DA(o), DA(Octree.from_numpy(m, 30, ctx=ctx))
    assert (da_h.n_elem, da_h.n_node) == (da_m.n_elem, da_m.n_node)
    x = np.ones(da_h.n_node)
    assert np.allclose(da_h.matvec(x).sum(), 1.0, atol=1e-12)


def test_batch_cloud_by_cloud(hctx, ctx, oracle):
    clouds = [datagen.gaussian(5000 + 1000 * i, 0.5, 0.1, seed=40 + i) for i in range(3)]
    hb = points2OctreeBatch(clouds, ctx=hctx)
    off = hb.segments()
    got = hb.to_numpy()
    for i, c in enumerate(clouds):
        want = oracle.hilbert_sort(points2Octree(c, ctx=ctx).to_numpy(), 30)
        assert np.array_equal(got[off[i]:off[i + 1]], want)


def test_files_in_hilbert_order(hctx, oracle, tmp_path):
    """Octree files written on a Hilbert context list the octants in the
    Hilbert build's order; reading them back gives the same octree."""
    from dendro_gb300 import readNodesFromFile, readNodesFromFile_binary, writeNodesToFile, writeNodesToFile_binary

    pts = datagen.lognormal(3000, seed=19)
    bal = balanceOctree(points2Octree(pts, ctx=hctx))
    want = bal.to_numpy()
    t, b = tmp_path / "h.ot", tmp_path / "h.otb"
    writeNodesToFile(str(t), bal)
    writeNodesToFile_binary(str(b), bal)
    lines = open(t).read().split("\n")
    rec = np.array([[int(v) for v in ln.split()] for ln in lines[2:] if ln.strip()], np.uint32)
    assert np.array_equal(rec, want)
    assert np.array_equal(readNodesFromFile(str(t), ctx=hctx).to_numpy(), want)
    assert np.array_equal(readNodesFromFile_binary(str(b), ctx=hctx).to_numpy(), want)
