"""completeOctree (src/construct.cpp:518): the oracle against the
reference's own outputs (tests/golden/ref_complete.npz, written by
tests/golden/make_golden.py from the reference code) and, on the inputs
where the reference aborts (an octant and a descendant in its first child:
getNCA's assertion, src/octFunctions.cpp:310), against the properties of a
completion.  CPU only."""
import os

import numpy as np
import pytest

from tests.golden import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ref():
    z = np.load(os.path.join(GOLDEN, "ref_complete.npz"))
    names = sorted({k.split("/")[0] for k in z.files})
    return {n: (z[f"{n}/in"], *(int(v) for v in z[f"{n}/params"]), z[f"{n}/out"], bool(z[f"{n}/aborted"]))
            for n in names}


def test_fixture_inputs_are_the_generated_ones(ref):
    gen = {name: (octs, D, u, s) for name, octs, D, u, s in cases.complete_inputs()}
    assert set(gen) == set(ref)
    for name, (octs, D, u, s, _, _) in ref.items():
        g = gen[name]
        assert np.array_equal(g[0].reshape(-1, 4), octs.reshape(-1, 4)) and (g[1], g[2], g[3]) == (D, u, s)


def test_oracle_matches_reference(ref, oracle):
    ran = 0
    for name, (octs, D, u, s, out, aborted) in ref.items():
        if aborted:
            continue
        got = oracle.complete(octs, D, u, s)
        assert np.array_equal(got, out.reshape(-1, 4)), name
        ran += 1
    assert ran >= 50


def _contains(a, b, D):
    """a[i] contains b[j] (or equals it), as an (len(a), len(b)) mask"""
    la = (1 << (D - a[:, 3].astype(np.int64)))[:, None]
    lb = (1 << (D - b[:, 3].astype(np.int64)))[None, :]
    ok = a[:, 3][:, None] <= b[:, 3][None, :]
    for c in range(3):
        ac, bc = a[:, c].astype(np.int64)[:, None], b[:, c].astype(np.int64)[None, :]
        ok &= (bc >= ac) & (bc + lb <= ac + la)
    return ok


def test_completion_properties(ref, oracle):
    """On every case (the reference's aborting ones included): the result is
    sorted, linear and complete, holds every input octant without a
    descendant in the input, and every other octant is as coarse as possible
    (its parent overlaps an input leaf)."""
    for name, (octs, D, u, s, _, _) in ref.items():
        got = oracle.complete(octs, D, u, s)
        if len(octs) == 0:
            assert len(got) == 0
            continue
        ch = oracle.checks(got, D)
        assert ch["sorted"] and ch["linear"] and ch["complete"], name
        uniq = np.unique(octs.reshape(-1, 4), axis=0)
        c = _contains(uniq, uniq, D)
        np.fill_diagonal(c, False)
        leaves = uniq[~c.any(axis=1)]
        got_set = {tuple(o) for o in got.tolist()}
        assert all(tuple(o) in got_set for o in leaves.tolist()), name
        fill = np.array([o for o in got.tolist() if tuple(o) not in {tuple(v) for v in leaves.tolist()}],
                        np.uint32).reshape(-1, 4)
        if len(fill):
            assert (fill[:, 3] > 0).all()
            par = fill.copy()
            par[:, 3] -= 1
            sh = (D - par[:, 3]).astype(np.uint64)
            for k in range(3):
                par[:, k] = ((par[:, k].astype(np.uint64) >> sh) << sh).astype(np.uint32)
            assert _contains(par, leaves, D).any(axis=1).all(), name


def test_some_reference_cases_abort(ref):
    """The fixture covers both the reference's completed and aborting inputs."""
    ab = [n for n, v in ref.items() if v[5]]
    assert 0 < len(ab) < len(ref) // 2
