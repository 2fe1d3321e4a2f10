"""Batched construction and balance: every cloud of a batch gets exactly the
octree the reference builds for it alone (the batching workload's rule)."""
import numpy as np
import pytest

from dendro_gb300 import DendroError, balanceOctree, datagen, points2Octree, points2OctreeBatch

pytestmark = pytest.mark.gpu


def make_batch(seed, count=24):
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = datagen.cloud_sizes(count, 1, 5e4, seed)
    clouds = [datagen.mixture(int(s), rng) for s in sizes]
    clouds[3] = np.zeros((0, 3))                     # empty cloud: the root
    clouds[5] = clouds[5][:1]                        # one point: the root
    clouds[7] = np.concatenate([clouds[7], clouds[7][:10]])  # repeated points
    return clouds


def test_batch_construct_matches_per_cloud_reference(ctx, oracle):
    clouds = make_batch(51)
    got = points2OctreeBatch(clouds, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
    parts = got.split()
    assert len(parts) == len(clouds)
    for c, part in zip(clouds, parts):
        ref = oracle.points_to_octree(c, 30, 1) if len(c) else np.zeros((1, 4), np.uint32)
        assert np.array_equal(part, ref)


def test_batch_balance_matches_per_cloud_reference(ctx, oracle):
    clouds = [c for i, c in enumerate(make_batch(52)) if i != 7]
    lin = points2OctreeBatch(clouds, ctx=ctx)
    bal = balanceOctree(lin)
    for c, part in zip(clouds, bal.split()):
        ref = oracle.balance(oracle.points_to_octree(c, 30, 1), 30) if len(c) else np.zeros((1, 4), np.uint32)
        assert np.array_equal(part, ref)


def test_same_alone_and_in_the_mix(ctx):
    clouds = make_batch(53, count=12)
    mix = balanceOctree(points2OctreeBatch(clouds, ctx=ctx)).split()
    for i in (0, 4, 9):
        alone = balanceOctree(points2Octree(clouds[i], ctx=ctx)).to_numpy() if len(clouds[i]) else None
        if alone is not None:
            assert np.array_equal(mix[i], alone)


@pytest.mark.parametrize("max_pts", [2, 7])
def test_batch_max_pts(ctx, oracle, max_pts):
    rng = np.random.Generator(np.random.PCG64(54))
    clouds = [datagen.gaussian(int(n), 0.5, 0.1, seed=int(n)) for n in rng.integers(1, 3000, 10)]
    parts = points2OctreeBatch(clouds, maxNumPtsPerOctant=max_pts, ctx=ctx).split()
    for c, part in zip(clouds, parts):
        assert np.array_equal(part, oracle.points_to_octree(c, 30, max_pts))


def test_batch_rejects_bad_offsets(ctx):
    pts = datagen.gaussian(100, seed=1)
    with pytest.raises(DendroError):
        points2OctreeBatch(pts, seg_start=np.array([0, 50, 40, 100], np.uint64), ctx=ctx)


def test_batch_of_device_tensors_equals_host_batch(ctx):
    """Clouds handed over as CUDA tensors (joined on the device by torch) give
    the same octrees as the same clouds from host memory, call after call:
    the library waits for torch's stream before it reads."""
    torch = pytest.importorskip("torch")
    clouds = [c for i, c in enumerate(make_batch(54, count=16)) if i != 7]
    want = [p.copy() for p in balanceOctree(points2OctreeBatch(clouds, ctx=ctx)).split()]
    dev = [torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in clouds]
    for _ in range(3):
        # scribble over freed torch memory so a read before the join completes shows
        junk = torch.full((sum(len(c) for c in clouds), 3), 0.25, dtype=torch.float64, device="cuda")
        del junk
        got = balanceOctree(points2OctreeBatch(dev, ctx=ctx)).split()
        for a, b in zip(want, got):
            assert np.array_equal(a, b)
