"""Per-element operators and diagonals on the GPU against the oracle:
Jacobian2MatMult (dg_matvec_coef), its assembled matrix
(dg_da_assemble_coef), Jacobian1/Jacobian2MatGetDiagonal (dg_da_diagonal)
and DirichletJacobianMatGetDiagonal (dg_mg_diagonal).  Tolerances: FP64
1e-12 of the result's largest entry (the GPU adds shared nodes' sums in
another order), FP32 relative L2 1e-6."""
import numpy as np
import pytest

from dendro_gb300 import DA, MultiGrid, balanceOctree, datagen, points2Octree

pytestmark = pytest.mark.gpu


def _perm(xyz_gpu, xyz_ref):
    og = np.lexsort(xyz_gpu.T[::-1])
    oo = np.lexsort(xyz_ref.T[::-1])
    assert np.array_equal(xyz_gpu[og], xyz_ref[oo])
    p = np.empty(len(oo), np.int64)
    p[oo] = og
    return p


@pytest.fixture(scope="module")
def mesh(ctx, oracle):
    pts = datagen.lognormal(30_000, seed=17)
    bal = balanceOctree(points2Octree(pts, ctx=ctx))
    da = DA(bal)
    oda = oracle.DA(bal.to_numpy(), 30)
    p = _perm(da.download()["node_xyz"], oda.node_xyz)
    coef = np.random.Generator(np.random.PCG64(8)).uniform(0.05, 4.0, (da.n_elem, 2))
    return da, oda, p, coef


def _close(got, want, tol):
    assert np.abs(got - want).max() <= tol * np.abs(want).max()


def test_matvec_coef(mesh, oracle):
    da, oda, p, coef = mesh
    x = np.random.Generator(np.random.PCG64(9)).uniform(-1, 1, oda.n_node)
    xg = np.empty_like(x)
    xg[p] = x
    want = oracle.matvec_coef(oda, coef, x)
    _close(da.matvec_coef(coef, xg)[p], want, 1e-12)
    y32 = da.matvec_coef(coef, xg.astype(np.float32), precision=32)[p].astype(np.float64)
    assert np.linalg.norm(y32 - want) <= 1e-6 * np.linalg.norm(want)
    # constant factors: the lapFac / massFac operator
    c = np.tile([0.7, 1.9], (da.n_elem, 1))
    _close(da.matvec_coef(c, xg), da.matvec(xg, lapFac=0.7, massFac=1.9), 1e-12)


def test_matvec_coef_device(mesh):
    torch = pytest.importorskip("torch")
    da, _, _, coef = mesh
    x = np.random.Generator(np.random.PCG64(10)).uniform(-1, 1, da.n_node)
    yd = da.matvec_coef(torch.from_numpy(coef).cuda(), torch.from_numpy(x).cuda())
    _close(yd.cpu().numpy(), da.matvec_coef(coef, x), 1e-12)


def test_diagonals(mesh, oracle):
    da, oda, p, coef = mesh
    _close(da.diagonal(0.3, 1.7)[p], oracle.diagonal(oda, 0.3, 1.7), 1e-12)
    _close(da.diagonal(coef=coef)[p], oracle.diagonal(oda, coef=coef), 1e-12)


def test_assembled_coef(mesh, oracle):
    da, oda, p, coef = mesh
    csr = da.assemble_coef(coef)
    ref = oracle.assemble(oda, coef=coef)
    g = csr.to_scipy()[p][:, p].tocsr()
    g.sort_indices()
    assert np.array_equal(g.indptr, ref.indptr) and np.array_equal(g.indices, ref.indices)
    _close(g.data, ref.data, 1e-12)
    x = np.random.Generator(np.random.PCG64(11)).uniform(-1, 1, da.n_node)
    _close(csr.spmv(x), da.matvec_coef(coef, x), 1e-12)


def test_mg_diagonal(ctx, oracle):
    pts = datagen.gaussian(4000, 0.5, 0.15, seed=3)
    mg = MultiGrid(balanceOctree(points2Octree(pts, ctx=ctx)), max_coarse_elems=600)
    for l in range(mg.n_levels):
        oda = oracle.DA(mg.level_octree(l), 30)
        p = _perm(mg.level_nodes(l), oda.node_xyz)
        _close(mg.diagonal(l)[p], oda.dirichlet_diag(), 1e-12)


def test_single_element_mesh(ctx, oracle):
    """The root octree: one element, eight nodes, a dense 8 x 8 matrix."""
    from dendro_gb300 import Octree

    root = np.array([[0, 0, 0, 0]], np.uint32)
    da = DA(Octree.from_numpy(root, 30, ctx=ctx))
    assert (da.n_elem, da.n_node) == (1, 8)
    oda = oracle.DA(root, 30)
    p = _perm(da.download()["node_xyz"], oda.node_xyz)
    csr = da.assemble(1.0, 1.0)
    assert csr.nnz == 64 and csr.max_row_len == 8
    g = csr.to_scipy()[p][:, p].toarray()
    _close(g, oracle.assemble(oda).toarray(), 1e-12)
    x = np.linspace(-1, 1, 8)
    _close(csr.spmv(x), da.matvec(x), 1e-12)
    coef = np.array([[3.0, 0.5]])
    xo = x[p]
    _close(da.matvec_coef(coef, x)[p], oracle.matvec_coef(oda, coef, xo), 1e-12)
    _close(da.diagonal(coef=coef)[p], oracle.diagonal(oda, coef=coef), 1e-12)
