"""Multigrid oracle checks (CPU): transfer stencils pinned to the reference's
RmatType1/2 tables, the transfers themselves pinned to the reference's own
restriction and prolongation loops, coarsening pinned to the reference,
P = R^T, and the restated PCG + V-cycle converging."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from dendro_gb300 import datagen
from oracle.mg_ref import OracleMG
from tests.golden import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_rmat_tables_match_reference(oracle):
    t = np.load(os.path.join(GOLDEN, "ref_tables.npz"))
    r1, r2 = oracle.rmat_tables()
    w = np.arange(1, 65, dtype=np.float64).reshape(8, 8)

    def stats(a):
        return np.stack([a.sum((-2, -1)), (a * w).sum((-2, -1)), (a * a).sum((-2, -1))], -1)

    assert np.allclose(stats(r1), t["rmat1_stats"], rtol=0, atol=1e-12)
    assert np.allclose(stats(r2), t["rmat2_stats"], rtol=0, atol=1e-12)


def test_coarsen_matches_reference_cases(oracle):
    g = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    bal = g["gauss3k/bal"]
    c = oracle.coarsen(bal, 30)
    assert oracle.checks(c, 30)["complete"] and oracle.checks(c, 30)["linear"]
    assert len(c) < len(bal)
    # coarsening never merges across a non-family: every parent output has 8 input children
    assert np.array_equal(oracle.coarsen(np.zeros((1, 4), np.uint32), 30), np.zeros((1, 4), np.uint32))


@pytest.fixture(scope="module")
def small_mg(oracle):
    pts = datagen.gaussian(2500, 0.5, 0.15, seed=3)
    bal = oracle.balance(oracle.points_to_octree(pts, 30, 1), 30)
    return OracleMG(bal, 30, max_coarse=400)


def test_transfers_are_adjoint(small_mg):
    rng = np.random.Generator(np.random.PCG64(2))
    for l in range(small_mg.n_levels - 1):
        u = rng.random(small_mg.das[l + 1].n_node)
        v = rng.random(small_mg.das[l].n_node)
        assert abs(v @ small_mg.prolong(l, u) - u @ small_mg.restrict(l, v)) <= 1e-12 * abs(v @ small_mg.prolong(l, u))


def test_prolongation_reproduces_coarse_linear_fields(small_mg):
    # a trilinear field on the coarse mesh is interpolated exactly at interior fine nodes
    for l in range(small_mg.n_levels - 1):
        xc = small_mg.das[l + 1].node_xyz.astype(np.float64) / (1 << 30)
        xf = small_mg.das[l].node_xyz.astype(np.float64) / (1 << 30)
        g = lambda x: 1.0 + 2 * x[:, 0] - x[:, 1] + 0.5 * x[:, 2]  # noqa: E731
        pf = small_mg.prolong(l, g(xc))
        interior = ~small_mg.das[l].bdy()
        ids, w = small_mg.pmaps[l]
        full = interior & np.isclose(w.sum(1), 1.0)
        assert np.allclose(pf[full], g(xf)[full], atol=1e-13)


def test_oracle_solver_converges(small_mg):
    b = small_mg.rhs(datagen.bumps(small_mg.das[0].node_xyz))
    x, it, rr = small_mg.solve(b, 1e-8, 100)
    assert rr <= 1e-8
    assert it < 30
    assert np.all(x[small_mg.das[0].bdy()] == 0.0)


@pytest.mark.parametrize("cloud", ["gaussian", "lognormal"])
def test_prolongation_weights_fit_the_packed_tables(oracle, small_mg, cloud):
    """The device keeps each nonzero prolongation weight as w * 64 in one
    byte, at most 8 per fine node: every weight of every level is a multiple
    of 1/64 in (0, 1] (shape-function values 1, 1/2, 1/4, 1/8 shared among
    at most 8 parent corners)."""
    if cloud == "gaussian":
        mg = small_mg
    else:
        pts = datagen.lognormal(3000, seed=7)
        mg = OracleMG(oracle.balance(oracle.points_to_octree(pts, 30, 1), 30), 30, max_coarse=300)
    assert mg.n_levels >= 3
    for l in range(mg.n_levels - 1):
        ids, w = mg.pmaps[l]
        nz = w[w != 0] * 64
        assert np.all(nz == np.round(nz)) and nz.min() >= 1 and nz.max() <= 64
        assert (w != 0).sum(1).max() <= 8
        assert np.all(ids[w != 0] < mg.das[l + 1].n_node)


@pytest.mark.parametrize("name", list(cases.TRANSFER))
def test_transfers_match_the_reference_loops(oracle, name):
    """The oracle's restriction and prolongation (the ones the GPU transfers
    are tested against) equal the reference's own restrictMatVecType1 and
    prolongMatVecType1 (src/omg/restrictMatVec.cpp, prolongMatVec.cpp, with
    the Dirichlet DOFs suppressed as SetDirichletJacContexts sets them), run
    by oracle/_ref/ref_driver between a balanced octree and its next coarser
    level: the same coarse level, and R v, P v at every node."""
    g = np.load(os.path.join(GOLDEN, "ref_mg_ops.npz"))
    fine, coarse = g[f"{name}/fine"], g[f"{name}/coarse"]
    assert np.array_equal(oracle.balance(oracle.coarsen(fine, 30), 30), coarse)
    fda, cda = oracle.DA(fine, 30), oracle.DA(coarse, 30)
    two = SimpleNamespace(pmaps=[fda.prolong_map(coarse, cda)], das=[fda, cda])
    r = OracleMG.restrict(two, 0, cases.hashed_nodal_values(fda.node_xyz))
    p = OracleMG.prolong(two, 0, cases.hashed_nodal_values(cda.node_xyz))
    for xyz, got, ref_xyz, ref in ((cda.node_xyz, r, g[f"{name}/r_xyz"], g[f"{name}/r"]),
                                   (fda.node_xyz, p, g[f"{name}/p_xyz"], g[f"{name}/p"])):
        mine, theirs = np.lexsort(xyz.T[::-1]), np.lexsort(ref_xyz.T[::-1])
        assert np.array_equal(xyz[mine], ref_xyz[theirs])
        assert np.abs(ref).max() > 0.1
        assert np.abs(got[mine] - ref[theirs]).max() <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("name", list(cases.TRANSFER))
def test_dirichlet_operator_matches_the_reference(oracle, name):
    """The oracle's Dirichlet level operator and its diagonal (the GPU's are
    tested against them) equal the reference's own DirichletJacobianMatMult
    and DirichletJacobianMatGetDiagonal (examples/src/backend/omgJac.C:958,
    1111, with SetDirichletJacContexts' boundary flags), run by
    oracle/_ref/ref_driver on the same octree: A v and diag(A) at every node
    to 1e-14 of the largest value (the sums run in another order)."""
    g = np.load(os.path.join(GOLDEN, "ref_mg_ops.npz"))
    da = oracle.DA(g[f"{name}/fine"], 30)
    av = da.dirichlet_matvec(cases.hashed_nodal_values(da.node_xyz))
    dg = da.dirichlet_diag()
    mine, theirs = np.lexsort(da.node_xyz.T[::-1]), np.lexsort(g[f"{name}/a_xyz"].T[::-1])
    assert np.array_equal(da.node_xyz[mine], g[f"{name}/a_xyz"][theirs])
    for got, ref in ((av, g[f"{name}/a"]), (dg, g[f"{name}/diag"])):
        assert np.abs(ref).max() > 0
        assert np.abs(got[mine] - ref[theirs]).max() <= 1e-14 * np.abs(ref).max()
    # boundary rows are the identity: diag 1 exactly, A v = v there
    bdy = g[f"{name}/diag"][theirs] == 1.0
    assert bdy.sum() > 0 and np.array_equal(av[mine][bdy], cases.hashed_nodal_values(da.node_xyz)[mine][bdy])


@pytest.mark.parametrize("name", [n for n, (_, lv) in cases.TRANSFER.items() if lv == 0])
def test_element_callbacks_match_the_reference(oracle, name):
    """The oracle's element-loop operators (the GPU's are tested against
    them) equal the reference's own MatShell callbacks, run by
    oracle/_ref/ref_driver on the same octree: Jacobian1MatMult /
    Jacobian1MatGetDiagonal and MassMatMult / MassMatGetDiagonal
    (examples/src/backend/odaJac.C:294,160,399,229), Jacobian2MatMult /
    Jacobian2MatGetDiagonal with per-element factors (omgJac.C:1776,1641).
    Tolerance 1e-12 of the largest value: the oracle's stencils come from
    their definition, the reference's from .inp files with 15 decimals."""
    from oracle import dg_oracle

    g = np.load(os.path.join(GOLDEN, "ref_mg_ops.npz"))
    fine = g[f"{name}/fine"]
    da = oracle.DA(fine, 30)
    assert np.array_equal(da.level, fine[:, 3])  # elements in octant order
    x = cases.hashed_nodal_values(da.node_xyz)
    coef = cases.element_factors(fine)
    want = {"j1": da.matvec(x), "j1d": dg_oracle.diagonal(da), "m": da.matvec(x, 0.0, 1.0),
            "md": dg_oracle.diagonal(da, 0.0, 1.0), "j2": dg_oracle.matvec_coef(da, coef, x),
            "j2d": dg_oracle.diagonal(da, coef=coef)}
    mine, theirs = np.lexsort(da.node_xyz.T[::-1]), np.lexsort(g[f"{name}/a_xyz"].T[::-1])
    assert np.array_equal(da.node_xyz[mine], g[f"{name}/a_xyz"][theirs])
    for op, got in want.items():
        ref = g[f"{name}/{op}"][theirs]
        assert np.abs(ref).max() > 0
        assert np.abs(got[mine] - ref).max() <= 1e-12 * np.abs(ref).max(), op
