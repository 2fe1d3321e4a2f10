"""The GPU's multigrid level operators and element-loop operators against
the reference's own (tests/golden/ref_mg_ops.npz, written by
tests/golden/make_golden.py from the reference's restrictMatVecType1,
prolongMatVecType1, DirichletJacobianMatMult / DirichletJacobianMatGetDiagonal,
Jacobian1MatMult / Jacobian1MatGetDiagonal, MassMatMult /
MassMatGetDiagonal and Jacobian2MatMult / Jacobian2MatGetDiagonal): FP64
results by node coordinates within 1e-12 of the largest value (the
reference's stencil files hold 15 decimals)."""
import os

import numpy as np
import pytest

import dendro_gb300 as dg
from tests.golden import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


def _same(xyz, got, ref_xyz, ref):
    mine, theirs = np.lexsort(xyz.T[::-1]), np.lexsort(ref_xyz.T[::-1])
    assert np.array_equal(xyz[mine], ref_xyz[theirs])
    assert np.abs(got[mine] - ref[theirs]).max() <= TOL * np.abs(ref).max()


@pytest.mark.parametrize("name", list(cases.TRANSFER))
def test_level_operators_match_the_reference(ctx, name):
    g = np.load(os.path.join(GOLDEN, "ref_mg_ops.npz"))
    fine, coarse = g[f"{name}/fine"], g[f"{name}/coarse"]
    # one coarsening: the next level holds exactly the reference's coarse octree
    mg = dg.MultiGrid(dg.Octree.from_numpy(fine, 30, ctx=ctx), max_coarse_elems=len(coarse))
    try:
        assert mg.n_levels == 2 and np.array_equal(mg.level_octree(1), coarse)
        fx, cx = mg.level_nodes(0), mg.level_nodes(1)
        _same(cx, mg.restrict(0, cases.hashed_nodal_values(fx)), g[f"{name}/r_xyz"], g[f"{name}/r"])
        _same(fx, mg.prolong(0, cases.hashed_nodal_values(cx)), g[f"{name}/p_xyz"], g[f"{name}/p"])
        _same(fx, mg.matvec(0, cases.hashed_nodal_values(fx)), g[f"{name}/a_xyz"], g[f"{name}/a"])
        _same(fx, mg.diagonal(0), g[f"{name}/a_xyz"], g[f"{name}/diag"])
    finally:
        mg.free()


@pytest.mark.parametrize("name", [n for n, (_, lv) in cases.TRANSFER.items() if lv == 0])
def test_element_operators_match_the_reference(ctx, name):
    g = np.load(os.path.join(GOLDEN, "ref_mg_ops.npz"))
    fine = g[f"{name}/fine"]
    da = dg.DA(dg.Octree.from_numpy(fine, 30, ctx=ctx))
    try:
        xyz = da.download()["node_xyz"]
        x = cases.hashed_nodal_values(xyz)
        coef = cases.element_factors(fine)  # elements in octree order
        got = {"j1": da.matvec(x), "j1d": da.diagonal(), "m": da.matvec(x, lapFac=0.0, massFac=1.0),
               "md": da.diagonal(0.0, 1.0), "j2": da.matvec_coef(coef, x), "j2d": da.diagonal(coef=coef)}
        for op, v in got.items():
            _same(xyz, v, g[f"{name}/a_xyz"], g[f"{name}/{op}"])
    finally:
        da.free()
