"""Assembled operators: the oracle's assembly (numpy) against the matrices
the reference itself assembles (CreateAndComputeFullJacobian1,
examples/src/backend/odaJac.C:470, through its DA and stencil files:
tests/golden/ref_mat.npz; and, called as the reference calls them with
entries through DA::setValuesInMatrix, CreateAndComputeFullJacobian1,
ComputeDirichletJacobian and ComputeJacobian2: tests/golden/ref_assemble.npz;
both written by tests/golden/make_golden.py).  The pattern must be
identical; the values agree to the precision of the reference's stencil
files (15 decimals).  CPU only."""
import os

import numpy as np
import pytest

from tests.golden import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _by_coords(m, node_xyz, ref_xyz):
    """rows / cols of a scipy matrix over node_xyz, re-indexed into ref_xyz"""
    key = lambda a: np.ascontiguousarray(a, np.uint32).view([("", np.uint32)] * 3).ravel()
    order = np.argsort(key(ref_xyz))
    pos = np.searchsorted(key(ref_xyz)[order], key(node_xyz))
    idx = order[pos]
    assert np.array_equal(ref_xyz[idx], node_xyz)
    c = m.tocoo()
    return idx[c.row], idx[c.col], c.data


def test_oracle_matches_reference_matrix(oracle):
    z = np.load(os.path.join(GOLDEN, "ref_mat.npz"))
    da = oracle.DA(z["bal"], 30)
    m = oracle.assemble(da)
    assert m.nnz == len(z["val"])
    r, c, v = _by_coords(m, da.node_xyz, z["node_xyz"])
    got = {(int(a), int(b)): x for a, b, x in zip(r, c, v)}
    ref = {(int(a), int(b)): x for a, b, x in zip(z["row"], z["col"], z["val"])}
    assert got.keys() == ref.keys()
    scale = np.abs(z["val"]).max()
    err = max(abs(got[k] - ref[k]) for k in ref) / scale
    assert err < 1e-12, err


def test_oracle_matrix_is_the_matvec(oracle):
    z = np.load(os.path.join(GOLDEN, "ref_mat.npz"))
    da = oracle.DA(z["bal"], 30)
    x = np.random.Generator(np.random.PCG64(3)).uniform(-1, 1, da.n_node)
    np.testing.assert_allclose(oracle.assemble(da, 0.7, 1.3) @ x, da.matvec(x, 0.7, 1.3), rtol=0, atol=1e-12)
    np.testing.assert_allclose(oracle.assemble(da, dirichlet=True) @ x, da.dirichlet_matvec(x), rtol=0, atol=1e-12)


def test_oracle_per_element_forms(oracle):
    """The per-element (Jacobian2) restatement with every element's factors
    equal to (a, b) is the C restatement of lapFac = a, massFac = b; its
    diagonal is the diagonal of its matrix."""
    z = np.load(os.path.join(GOLDEN, "ref_mat.npz"))
    da = oracle.DA(z["bal"], 30)
    x = np.random.Generator(np.random.PCG64(5)).uniform(-1, 1, da.n_node)
    coef = np.tile([0.4, 2.5], (da.n_elem, 1))
    np.testing.assert_allclose(oracle.matvec_coef(da, coef, x), da.matvec(x, 0.4, 2.5), rtol=0, atol=1e-13)
    rc = np.random.Generator(np.random.PCG64(6)).uniform(0.1, 3.0, (da.n_elem, 2))
    m = oracle.assemble(da, coef=rc)
    np.testing.assert_allclose(m @ x, oracle.matvec_coef(da, rc, x), rtol=0, atol=1e-13)
    np.testing.assert_allclose(m.diagonal(), oracle.diagonal(da, coef=rc), rtol=0, atol=1e-15)


@pytest.mark.parametrize("name", list(cases.ASSEMBLE))
def test_oracle_matches_reference_assembly_functions(oracle, name):
    """K + M, the Dirichlet matrix and the per-element-factor matrix of the
    oracle (which the GPU's CSR assembly is tested against) summarised as the
    reference's own CreateAndComputeFullJacobian1, ComputeDirichletJacobian
    (examples/src/backend/omgJac.C:383) and ComputeJacobian2 (omgJac.C:1861)
    are: the same pattern and entry count, and A v, A 1 and diag(A) to 1e-12
    of their largest values."""
    z = np.load(os.path.join(GOLDEN, "ref_assemble.npz"))
    bal = z[f"{name}/bal"]
    da = oracle.DA(bal, 30)
    key = lambda a: np.ascontiguousarray(a, np.uint32).view([("", np.uint32)] * 3).ravel()
    assert np.array_equal(np.sort(key(da.node_xyz)), key(z[f"{name}/node_xyz"]))
    mats = {"k": oracle.assemble(da), "kd": oracle.assemble(da, dirichlet=True),
            "k2": oracle.assemble(da, coef=cases.element_factors(bal))}
    for m, a in mats.items():
        c = a.tocoo()
        got = cases.csr_summary(da.node_xyz, c.row, c.col, c.data)
        assert int(got["nnz"]) == int(z[f"{name}/{m}/nnz"]), m
        assert got["pattern"] == str(z[f"{name}/{m}/pattern"]), m
        for k in ("av", "a1", "diag"):
            ref = z[f"{name}/{m}/{k}"]
            assert np.abs(got[k] - ref).max() <= 1e-12 * np.abs(ref).max(), (m, k)
