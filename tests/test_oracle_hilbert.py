"""Hilbert order (the reference's default build, -DHILBERT_ORDERING): the
oracle's restatement of the Hilbert comparison (TreeNode::operator<,
include/TreeNode.tcc:130-210) against outputs of the reference's own
Hilbert build (tests/golden/ref_hilbert.npz, written by
tests/golden/make_golden.py).  The Hilbert build makes the same octants as
the Morton build; only their order differs.  CPU only."""
import os

import numpy as np
import pytest

from tests.golden import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fnv1a(o):
    h = 1469598103934665603
    for byte in np.ascontiguousarray(o, np.uint32).tobytes():
        h ^= byte
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


@pytest.fixture(scope="module")
def hil():
    return np.load(os.path.join(GOLDEN, "ref_hilbert.npz"))


@pytest.fixture(scope="module")
def morton():
    return np.load(os.path.join(GOLDEN, "ref_cases.npz"))


def _same(got, z, key):
    assert len(got) == int(z[f"{key}_n"]), key
    assert fnv1a(got) == int(z[f"{key}_fnv"]), key
    full = z[key].reshape(-1, 4)
    if len(full):
        assert np.array_equal(got, full), key


def test_curve_tables(oracle):
    assert oracle.hilbert_states() == 24


def test_points_cases(hil, morton, oracle):
    """Hilbert order of the Morton build's construction and balance outputs
    = the Hilbert build's outputs, case by case."""
    ran = 0
    for name in cases.SMALL:
        if not bool(hil[f"p2o_{name}/finished"]):
            continue
        D = int(hil[f"p2o_{name}/params"][0])
        if (morton[f"{name}/lin"].astype(np.uint64)[:, :3] >> D).any():
            continue  # octants outside the domain (repeated points): no Hilbert position
        _same(oracle.hilbert_sort(morton[f"{name}/lin"], D), hil, f"p2o_{name}/lin")
        bal = morton[f"{name}/bal"].reshape(-1, 4)
        if len(bal) or int(morton[f"{name}/bal_n"]) == 0:
            _same(oracle.hilbert_sort(bal, D), hil, f"p2o_{name}/bal")
        ran += 1
    assert ran >= 7


def test_complete_cases(hil, oracle):
    ran = 0
    for name, octs, D, u, s in cases.complete_inputs():
        key = f"complete_{name}"
        if f"{key}/finished" not in hil.files or not bool(hil[f"{key}/finished"]):
            continue
        _same(oracle.hilbert_sort(oracle.complete(octs, D, 0, 0), D), hil, f"{key}/out")
        ran += 1
    assert ran >= 20


def test_hilbert_sort_is_a_total_order(oracle):
    """Sorting is independent of the input order, keeps ancestors before
    their descendants, and sorting twice changes nothing."""
    rng = np.random.Generator(np.random.PCG64(9))
    octs = cases.morton_sort(cases.sparse_octants(rng, 10, 5, keep=0.5, n_anc=30), 10)
    a = oracle.hilbert_sort(octs, 10)
    sh = octs.copy()
    rng.shuffle(sh)
    assert np.array_equal(oracle.hilbert_sort(sh, 10), a)
    assert np.array_equal(oracle.hilbert_sort(a, 10), a)
    pos = {tuple(o): i for i, o in enumerate(a.tolist())}
    for x, y, z, lev in a.tolist():
        for la in range(lev):
            m = ~((1 << (10 - la)) - 1) & 0xFFFFFFFF
            anc = (x & m, y & m, z & m, la)
            if anc in pos:
                assert pos[anc] < pos[(x, y, z, lev)]
