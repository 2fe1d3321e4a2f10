"""Multigrid slice on the GPU against the oracle: level octrees (coarsen +
balance chain) bit-exact, Dirichlet operator and transfers per level within
the FP64 / FP32 tolerances, and the FP32- and FP64-preconditioned CG solves
reaching 1e-8 relative residual with the oracle's solution."""
import numpy as np
import pytest

from dendro_gb300 import DendroError, MultiGrid, Octree, balanceOctree, coarsenOctree, datagen, points2Octree
from oracle.mg_ref import OracleMG

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12
FP32_RTOL = 1e-6


def _perm(xyz_gpu, xyz_ref):
    """p with xyz_gpu[p[i]] == xyz_ref[i]"""
    og = np.lexsort(xyz_gpu.T[::-1])
    oo = np.lexsort(xyz_ref.T[::-1])
    assert np.array_equal(xyz_gpu[og], xyz_ref[oo])
    p = np.empty(len(oo), np.int64)
    p[oo] = og
    return p


@pytest.fixture(scope="module")
def problem(oracle):
    pts = datagen.gaussian(4000, 0.5, 0.15, seed=3)
    bal = oracle.balance(oracle.points_to_octree(pts, 30, 1), 30)
    return bal, OracleMG(bal, 30, max_coarse=600)


def test_coarsen_matches_oracle(ctx, oracle, problem):
    bal, _ = problem
    got = coarsenOctree(Octree.from_numpy(bal, 30, ctx=ctx)).to_numpy()
    assert np.array_equal(got, oracle.coarsen(bal, 30))


def test_levels_match_oracle(ctx, problem):
    bal, ref = problem
    mg = MultiGrid(Octree.from_numpy(bal, 30, ctx=ctx), max_coarse_elems=600)
    assert mg.n_levels == ref.n_levels
    for l in range(mg.n_levels):
        assert np.array_equal(mg.level_octree(l), ref.octs[l])
        assert mg.sizes[l] == (ref.das[l].n_elem, ref.das[l].n_node)


def test_level_operators(ctx, problem):
    bal, ref = problem
    mg = MultiGrid(Octree.from_numpy(bal, 30, ctx=ctx), max_coarse_elems=600)
    rng = np.random.Generator(np.random.PCG64(5))
    perms = [_perm(mg.level_nodes(l), ref.das[l].node_xyz) for l in range(mg.n_levels)]
    for l in range(mg.n_levels):
        p = perms[l]
        x = rng.uniform(-1, 1, ref.das[l].n_node)
        xg = np.empty_like(x)
        xg[p] = x
        y_ref = ref.matvec(l, x)
        y64 = mg.matvec(l, xg, precision=64)[p]
        assert np.linalg.norm(y64 - y_ref) <= FP64_RTOL * np.linalg.norm(y_ref)
        y32 = mg.matvec(l, xg.astype(np.float32), precision=32)[p]
        assert np.linalg.norm(y32 - y_ref) <= FP32_RTOL * np.linalg.norm(y_ref)
        if l + 1 < mg.n_levels:
            pc = perms[l + 1]
            r_ref = ref.restrict(l, x)
            r64 = mg.restrict(l, xg, precision=64)[pc]
            assert np.linalg.norm(r64 - r_ref) <= FP64_RTOL * np.linalg.norm(r_ref)
            xc = rng.uniform(-1, 1, ref.das[l + 1].n_node)
            xcg = np.empty_like(xc)
            xcg[pc] = xc
            p_ref = ref.prolong(l, xc)
            p64 = mg.prolong(l, xcg, precision=64)[p]
            assert np.linalg.norm(p64 - p_ref) <= FP64_RTOL * np.linalg.norm(p_ref)
            p32 = mg.prolong(l, xcg.astype(np.float32), precision=32)[p]
            assert np.linalg.norm(p32 - p_ref) <= FP32_RTOL * np.linalg.norm(p_ref)


@pytest.mark.parametrize("precision", [64, 32])
def test_solve_matches_oracle(ctx, problem, precision):
    bal, ref = problem
    mg = MultiGrid(Octree.from_numpy(bal, 30, ctx=ctx), max_coarse_elems=600)
    p = _perm(mg.level_nodes(0), ref.das[0].node_xyz)
    f_ref = datagen.bumps(ref.das[0].node_xyz)
    b_ref = ref.rhs(f_ref)
    x_ref, it_ref, rr_ref = ref.solve(b_ref, 1e-8, 200)
    assert rr_ref <= 1e-8
    f = datagen.bumps(mg.level_nodes(0))
    b = mg.rhs(f)
    assert np.linalg.norm(b[p] - b_ref) <= FP64_RTOL * np.linalg.norm(b_ref)
    x, it, rr = mg.solve(b, precision=precision, rtol=1e-8, maxit=200)
    assert rr <= 1e-8
    assert it <= it_ref + 3
    assert np.linalg.norm(x[p] - x_ref) <= 1e-6 * np.linalg.norm(x_ref)
    # boundary values stay zero (Dirichlet u = 0)
    xyz = mg.level_nodes(0)
    on_bdy = np.any((xyz == 0) | (xyz == (1 << 30)), axis=1)
    assert np.all(x[on_bdy] == 0.0)


def test_solve_larger_cloud_both_precisions(ctx):
    pts = datagen.gaussian(200_000, 0.5, 0.15, seed=3)
    bal = balanceOctree(points2Octree(pts, ctx=ctx))
    mg = MultiGrid(bal, max_coarse_elems=4096)
    b = mg.rhs(datagen.bumps(mg.level_nodes(0)))
    x64, it64, rr64 = mg.solve(b, precision=64)
    x32, it32, rr32 = mg.solve(b, precision=32)
    assert rr64 <= 1e-8 and rr32 <= 1e-8
    assert abs(it32 - it64) <= 3
    assert np.linalg.norm(x32 - x64) <= 1e-6 * np.linalg.norm(x64)


def test_mg_rejects_batches(ctx):
    from dendro_gb300 import points2OctreeBatch

    lin = points2OctreeBatch([datagen.gaussian(100, seed=1), datagen.gaussian(100, seed=2)], ctx=ctx)
    with pytest.raises(DendroError) as e:
        MultiGrid(balanceOctree(lin))
    assert e.value.status == 9


@pytest.mark.parametrize("npts", [3, 40, 500, 700])
def test_single_level_is_an_exact_coarse_solve(ctx, oracle, npts):
    """With one level the V-cycle is the coarsest solve itself (block
    Gauss-Jordan FP32 inverse, FP64 refinement rounds): CG stops after one
    iteration, and the solution equals the oracle's dense FP64 solve.  The
    sizes put the coarse operator below one 64-wide block, across a few
    blocks and with a partial last block."""
    from oracle.mg_ref import OracleMG

    bal = oracle.balance(oracle.points_to_octree(datagen.gaussian(npts, 0.5, 0.2, seed=npts), 30, 1), 30)
    mg = MultiGrid(Octree.from_numpy(bal, 30, ctx=ctx), max_coarse_elems=len(bal))
    assert mg.n_levels == 1
    b = mg.rhs(datagen.bumps(mg.level_nodes(0)))
    ref = OracleMG(bal, 30, max_coarse=len(bal))
    p = _perm(mg.level_nodes(0), ref.das[0].node_xyz)
    x_ref = ref.cinv @ ref.rhs(datagen.bumps(ref.das[0].node_xyz))
    # FP64 V-cycle: the preconditioner is the exact inverse, one iteration;
    # FP32 V-cycle: its output is rounded to FP32, so one more iteration
    for precision, iters in ((64, 1), (32, 2)):
        x, it, rr = mg.solve(b, precision=precision, rtol=1e-10, maxit=5)
        assert it <= iters and rr <= 1e-10, (precision, it, rr)
        assert np.linalg.norm(x[p] - x_ref) <= 1e-9 * np.linalg.norm(x_ref)


def test_fp32_cg_operator_with_reliable_updates(ctx):
    """The FP32 CG operator (dg_mg_set_cg_operator(32)): the recurrence
    residual is replaced by the FP64 one, so the solve still stops at an FP64
    relative residual of 1e-8 and agrees with the FP64-operator solve."""
    pts = datagen.gaussian(200_000, 0.5, 0.15, seed=3)
    bal = balanceOctree(points2Octree(pts, ctx=ctx))
    mg = MultiGrid(bal, max_coarse_elems=4096)
    b = mg.rhs(datagen.bumps(mg.level_nodes(0)))
    x64, it64, rr64 = mg.solve(b, precision=32)
    mg.set_cg_operator(32, 1e-3)
    x32, it32, rr32 = mg.solve(b, precision=32)
    assert rr64 <= 1e-8 and rr32 <= 1e-8
    assert it32 <= it64 + 4
    assert np.linalg.norm(x32 - x64) <= 1e-6 * np.linalg.norm(x64)
    with pytest.raises(DendroError):
        mg.set_cg_operator(16)


def test_double_single_operator(ctx):
    """The double-single level operator (precision 48: FP64 vectors, FP32-pair
    arithmetic) agrees with the FP64 operator to 1e-12 of its norm, and a
    solve with it as the CG operator reaches the same FP64 relative residual
    in the same number of iterations (within one) as the FP64 operator."""
    pts = datagen.gaussian(200_000, 0.5, 0.15, seed=3)
    bal = balanceOctree(points2Octree(pts, ctx=ctx))
    mg = MultiGrid(bal, max_coarse_elems=4096)
    rng = np.random.Generator(np.random.PCG64(21))
    for level in range(min(mg.n_levels, 3)):
        x = rng.uniform(-1.0, 1.0, mg.sizes[level][1])
        y64 = mg.matvec(level, x, precision=64)
        y48 = mg.matvec(level, x, precision=48)
        assert np.linalg.norm(y48 - y64) <= FP64_RTOL * np.linalg.norm(y64), level
    # magnitudes far from one: the loop scales x by a power of two to keep
    # its FP32 parts away from FP32's underflow and overflow
    x = rng.uniform(-1.0, 1.0, mg.sizes[0][1])
    for scale in (1e-30, 1e-12, 1e25):
        y64 = mg.matvec(0, x * scale, precision=64)
        y48 = mg.matvec(0, x * scale, precision=48)
        assert np.linalg.norm(y48 - y64) <= FP64_RTOL * np.linalg.norm(y64), scale
    # a smooth field: the Laplacian cancels, the rows' terms are large
    # against the result
    xs = datagen.bumps(mg.level_nodes(0))
    y64 = mg.matvec(0, xs, precision=64)
    y48 = mg.matvec(0, xs, precision=48)
    assert np.linalg.norm(y48 - y64) <= 1e-10 * np.linalg.norm(y64)
    b = mg.rhs(datagen.bumps(mg.level_nodes(0)))
    for bscale in (1.0, 1e-25):  # a tiny right-hand side (fine meshes' loads are of order h^3)
        mg.set_cg_operator(64)
        x64, it64, rr64 = mg.solve(b * bscale, precision=32)
        mg.set_cg_operator(48)  # the default
        x48, it48, rr48 = mg.solve(b * bscale, precision=32)
        assert rr64 <= 1e-8 and rr48 <= 1e-8, bscale
        assert abs(it48 - it64) <= 1, bscale
        assert np.linalg.norm(x48 - x64) <= 1e-7 * np.linalg.norm(x64), bscale
