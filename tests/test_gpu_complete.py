"""completeOctree on the GPU (dg_complete_octree through the C ABI) against
the reference's outputs (tests/golden/ref_complete.npz) and the oracle:
bit-exact octants, host and device inputs, large sparse inputs at
maxDepth 30, and the error cases."""
import os

import numpy as np
import pytest

from dendro_gb300 import DendroError, balanceOctree, completeOctree, datagen, points2Octree
from tests.golden import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DG_ERR_INVALID_ARG, DG_ERR_DOMAIN = 1, 4


def test_golden_cases(ctx, oracle):
    z = np.load(os.path.join(GOLDEN, "ref_complete.npz"))
    names = sorted({k.split("/")[0] for k in z.files})
    for n in names:
        octs = z[f"{n}/in"].reshape(-1, 4)
        D, u, s = (int(v) for v in z[f"{n}/params"])
        got = completeOctree(octs, D, bool(u), bool(s), ctx=ctx).to_numpy()
        if not bool(z[f"{n}/aborted"]):
            assert np.array_equal(got, z[f"{n}/out"].reshape(-1, 4)), n
        # every case, the reference's aborting inputs included: the oracle
        assert np.array_equal(got, oracle.complete(octs, D, u, s)), n


@pytest.mark.parametrize("D,lmax,keep,n_anc,n_dup", [(30, 7, 0.2, 50, 1000), (30, 9, 0.02, 0, 0),
                                                     (12, 6, 0.5, 200, 5000), (4, 4, 0.7, 5, 10)])
def test_large_against_oracle(ctx, oracle, D, lmax, keep, n_anc, n_dup):
    rng = np.random.Generator(np.random.PCG64(D * 100 + lmax))
    octs = cases.sparse_octants(rng, D, lmax, keep=keep, p_split=0.7, n_anc=n_anc, n_dup=n_dup)
    want = oracle.complete(octs, D, 0, 0)
    assert np.array_equal(completeOctree(octs, D, ctx=ctx).to_numpy(), want)
    srt = np.unique(octs, axis=0)  # unique, not in Morton order
    assert np.array_equal(completeOctree(srt, D, isUnique=True, ctx=ctx).to_numpy(), oracle.complete(srt, D, 1, 0))


def test_device_input_and_idempotence(ctx, oracle):
    torch = pytest.importorskip("torch")
    pts = datagen.lognormal(200_000, seed=7)
    lin = points2Octree(pts, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
    bal = balanceOctree(lin)
    a = bal.to_numpy()
    dev = torch.from_numpy(a.view(np.int32)).to("cuda:0")
    # a sorted, linear, complete octree is its own completion
    assert np.array_equal(completeOctree(dev, 30, True, True, ctx=ctx).to_numpy(), a)
    # every 7th octant, shuffled, from device memory
    sub = a[::7].copy()
    np.random.Generator(np.random.PCG64(1)).shuffle(sub)
    got = completeOctree(torch.from_numpy(sub.view(np.int32)).to("cuda:0"), 30, ctx=ctx).to_numpy()
    assert np.array_equal(got, oracle.complete(sub, 30, 0, 0))


def test_edge_and_error_cases(ctx):
    assert completeOctree(np.zeros((0, 4), np.uint32), 30, ctx=ctx).size == 0
    assert completeOctree(np.array([[0, 0, 0, 0]], np.uint32), 30, ctx=ctx).to_numpy().tolist() == [[0, 0, 0, 0]]
    with pytest.raises(DendroError) as e:  # anchor not aligned to its level
        completeOctree(np.array([[2, 0, 0, 2]], np.uint32), 4, ctx=ctx)
    assert e.value.status == DG_ERR_DOMAIN
    with pytest.raises(DendroError) as e:  # level above maxDepth
        completeOctree(np.array([[0, 0, 0, 5]], np.uint32), 4, ctx=ctx)
    assert e.value.status == DG_ERR_DOMAIN
    unsorted = np.array([[8, 0, 0, 1], [0, 0, 0, 1]], np.uint32)
    with pytest.raises(DendroError) as e:  # declared sorted, is not
        completeOctree(unsorted, 4, True, True, ctx=ctx)
    assert e.value.status == DG_ERR_INVALID_ARG
    with pytest.raises(DendroError) as e:  # declared unique, is not
        completeOctree(np.array([[0, 0, 0, 1], [0, 0, 0, 1]], np.uint32), 4, True, True, ctx=ctx)
    assert e.value.status == DG_ERR_INVALID_ARG
    # the context stays usable after the errors
    assert completeOctree(unsorted, 4, ctx=ctx).size == 8


def test_sort_octants(ctx, oracle):
    """par::sampleSort / par::removeDuplicates of octant records: the
    oracle's Morton order (repeats kept or removed), and the Hilbert order
    on a Hilbert context."""
    from dendro_gb300 import Context, sortOctants

    rng = np.random.Generator(np.random.PCG64(31))
    octs = cases.sparse_octants(rng, 30, 7, keep=0.3, n_anc=40, n_dup=500)
    uniq = cases.morton_sort(octs, 30)
    assert np.array_equal(sortOctants(octs, 30, True, ctx=ctx), uniq)
    got = sortOctants(octs, 30, False, ctx=ctx)
    assert len(got) == len(octs)
    assert np.array_equal(np.unique(got, axis=0), np.unique(octs, axis=0))
    assert np.array_equal(got[np.r_[True, np.any(got[1:] != got[:-1], axis=1)]], uniq)
    h = Context(0)
    try:
        h.set_order("hilbert")
        assert np.array_equal(sortOctants(octs, 30, True, ctx=h), oracle.hilbert_sort(uniq, 30))
    finally:
        h.close()
