"""Assembled operators on the GPU (dg_da_assemble, dg_mg_assemble,
dg_csr_spmv) against the reference's assembled matrix
(tests/golden/ref_mat.npz) and the oracle's assembly: identical sparsity
patterns (sorted columns), values within FP64 rounding of the oracle, and
A x equal to the matrix-free operator."""
import os

import numpy as np
import pytest

from dendro_gb300 import DA, MultiGrid, Octree, balanceOctree, datagen, points2Octree

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL = 1e-12  # relative to the largest entry; the sums run in the same element order


def _perm(xyz_gpu, xyz_ref):
    """p with xyz_gpu[p[i]] == xyz_ref[i]"""
    og = np.lexsort(xyz_gpu.T[::-1])
    oo = np.lexsort(xyz_ref.T[::-1])
    assert np.array_equal(xyz_gpu[og], xyz_ref[oo])
    p = np.empty(len(oo), np.int64)
    p[oo] = og
    return p


def _check(csr, ref, p):
    """csr (GPU node ids) equals the scipy matrix ref (ids of the reference
    node list) under node permutation p"""
    rp, col, val = csr.to_numpy()
    assert csr.n_rows == ref.shape[0] and csr.nnz == ref.nnz
    for r in range(csr.n_rows):  # sorted columns in every row
        assert np.all(np.diff(col[rp[r]:rp[r + 1]].astype(np.int64)) > 0)
    inv = np.empty_like(p)
    inv[p] = np.arange(len(p))
    g = csr.to_scipy()[p][:, p].tocsr()
    g.sort_indices()
    ref = ref.tocsr()
    ref.sort_indices()
    assert np.array_equal(g.indptr, ref.indptr) and np.array_equal(g.indices, ref.indices)
    scale = np.abs(ref.data).max()
    assert np.abs(g.data - ref.data).max() <= RTOL * scale


def test_reference_matrix(ctx):
    import scipy.sparse as sp

    z = np.load(os.path.join(GOLDEN, "ref_mat.npz"))
    da = DA(Octree.from_numpy(z["bal"], 30, ctx=ctx))
    csr = da.assemble()
    n = len(z["node_xyz"])
    ref = sp.coo_matrix((z["val"], (z["row"].astype(np.int64), z["col"].astype(np.int64))), shape=(n, n)).tocsr()
    _check(csr, ref, _perm(da.download()["node_xyz"], z["node_xyz"]))
    assert 1 <= csr.max_row_len <= 128


@pytest.mark.parametrize("npts,lap,mass", [(3000, 1.0, 1.0), (30000, 0.5, 2.0)])
def test_against_oracle_and_matvec(ctx, oracle, npts, lap, mass):
    pts = datagen.lognormal(npts, seed=npts)
    bal = balanceOctree(points2Octree(pts, ctx=ctx))
    da = DA(bal)
    csr = da.assemble(lap, mass)
    oda = oracle.DA(bal.to_numpy(), 30)
    _check(csr, oracle.assemble(oda, lap, mass), _perm(da.download()["node_xyz"], oda.node_xyz))
    x = np.random.Generator(np.random.PCG64(1)).uniform(-1, 1, da.n_node)
    np.testing.assert_allclose(csr.spmv(x), da.matvec(x, lapFac=lap, massFac=mass), rtol=0, atol=1e-12)


def test_multigrid_levels(ctx, oracle):
    pts = datagen.gaussian(4000, 0.5, 0.15, seed=3)
    bal = balanceOctree(points2Octree(pts, ctx=ctx))
    mg = MultiGrid(bal, max_coarse_elems=600)
    rng = np.random.Generator(np.random.PCG64(2))
    for l in range(mg.n_levels):
        csr = mg.assemble(l)
        oda = oracle.DA(mg.level_octree(l), 30)
        _check(csr, oracle.assemble(oda, dirichlet=True), _perm(mg.level_nodes(l), oda.node_xyz))
        x = rng.uniform(-1, 1, csr.n_rows)
        np.testing.assert_allclose(csr.spmv(x), mg.matvec(l, x, precision=64), rtol=0, atol=1e-12)


def test_device_spmv(ctx):
    torch = pytest.importorskip("torch")
    da = DA(balanceOctree(points2Octree(datagen.gaussian(20000, 0.5, 0.1, seed=8), ctx=ctx)))
    csr = da.assemble()
    x = torch.rand(da.n_node, dtype=torch.float64, device="cuda:0")
    y = csr.spmv(x)
    np.testing.assert_allclose(y.cpu().numpy(), csr.spmv(x.cpu().numpy()), rtol=0, atol=0)


def test_compressed_da(ctx):
    """compressLut: same element data, node list, matVec and matrix, in less
    device memory."""
    pts = datagen.lognormal(60_000, seed=21)
    bal = balanceOctree(points2Octree(pts, ctx=ctx))
    plain, comp = DA(bal), DA(bal, compressLut=True)
    dp, dc = plain.download(), comp.download()
    for k in dp:
        assert np.array_equal(dp[k], dc[k]), k
    x = np.random.Generator(np.random.PCG64(4)).uniform(-1, 1, plain.n_node)
    # the element loop adds shared nodes' sums atomically: equal to rounding
    np.testing.assert_allclose(comp.matvec(x), plain.matvec(x), rtol=1e-12, atol=1e-15)
    x32 = x.astype(np.float32)
    np.testing.assert_allclose(comp.matvec(x32, precision=32), plain.matvec(x32, precision=32), rtol=1e-4, atol=1e-7)
    a, b = plain.assemble().to_numpy(), comp.assemble().to_numpy()
    assert all(np.array_equal(u, v) for u, v in zip(a, b))
    assert comp.memory_bytes() < 0.7 * plain.memory_bytes()
