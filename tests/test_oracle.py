"""The oracle pinned against the reference's own outputs (CPU only).

tests/golden holds outputs of the reference code itself (built from its
sources by oracle/Makefile, generated by tests/golden/make_golden.py); the
oracle's C restatement must reproduce them exactly.
"""
import json
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
def ref_cases():
    return np.load(os.path.join(GOLDEN, "ref_cases.npz"))


@pytest.mark.parametrize("name", sorted(cases.SMALL))
def test_points2octree_matches_reference(oracle, ref_cases, name):
    depth, maxpts = (int(v) for v in ref_cases[f"{name}/params"])
    pts = ref_cases[f"{name}/pts"]
    # the committed inputs are the generator's output
    assert np.array_equal(pts, cases.SMALL[name][0]())
    got = oracle.points_to_octree(pts, depth, maxpts)
    assert np.array_equal(got, ref_cases[f"{name}/lin"])


@pytest.mark.parametrize("name", sorted(cases.SMALL))
def test_balance_matches_reference(oracle, ref_cases, name):
    if bool(ref_cases[f"{name}/bal_aborted"]):
        pytest.skip("the reference aborts on this input (octants outside the domain)")
    depth = int(ref_cases[f"{name}/params"][0])
    got = oracle.balance(ref_cases[f"{name}/lin"], depth)
    assert len(got) == int(ref_cases[f"{name}/bal_n"])
    assert fnv1a(got) == int(ref_cases[f"{name}/bal_fnv"])
    if len(ref_cases[f"{name}/bal"]):
        assert np.array_equal(got, ref_cases[f"{name}/bal"])
    c = oracle.checks(got, depth)
    assert all(c.values()), c


def test_reference_quirk_out_of_domain_octants(ref_cases):
    """Repeated points can drive the reference's construction walk past the
    root: its output then holds octants outside the domain."""
    lin = ref_cases["boundary1500/lin"]
    assert (lin[:, :3] >= (1 << 30)).any()


@pytest.mark.parametrize("name", ["gauss20k", "lognormal100k"])
def test_larger_cases_hashes(oracle, name):
    exp = json.load(open(os.path.join(GOLDEN, "ref_hashes.json")))[name]
    fn, depth, maxpts = cases.LARGE[name]
    lin = oracle.points_to_octree(fn(), depth, maxpts)
    assert len(lin) == exp["n_lin"]
    assert f"{fnv1a(lin):016x}" == exp["fnv_lin"]
    bal = oracle.balance(lin, depth)
    assert len(bal) == exp["n_bal"]
    assert f"{fnv1a(bal):016x}" == exp["fnv_bal"]


def test_etype_table_matches_reference(oracle):
    t = np.load(os.path.join(GOLDEN, "ref_tables.npz"))
    assert np.array_equal(oracle.etype_masks(), t["etype_masks"])


def test_stencils_match_reference_tables(oracle):
    t = np.load(os.path.join(GOLDEN, "ref_tables.npz"))
    lap, mass = oracle.stencils()
    w = np.arange(1, 65, dtype=np.float64).reshape(8, 8)

    def stats(a):
        return np.stack([a.sum((2, 3)), (a * a).sum((2, 3)), (a * w).sum((2, 3)), a[:, :, 0, :].sum(2)], -1)

    # the reference tables are printed with 15 decimals
    assert np.allclose(stats(lap), t["lap_stats"], rtol=0, atol=1e-12)
    assert np.allclose(stats(mass), t["mass_stats"], rtol=0, atol=1e-12)
    # symmetric, rows of the Laplacian sum to zero for the conforming type
    assert np.allclose(lap, lap.transpose(0, 1, 3, 2))
    assert np.allclose(lap[:, 0].sum(-1), 0.0, atol=1e-14)


def test_da_matches_reference(oracle):
    g = np.load(os.path.join(GOLDEN, "ref_da.npz"))
    da = oracle.DA(g["bal"], 30)
    assert da.n_elem == len(g["bal"])
    assert da.n_node == int(g["n_nodes"])
    assert np.array_equal(da.level + 1, g["level"])  # the DA embeds one level deeper
    assert np.array_equal(da.child, g["child"])
    assert np.array_equal(da.hmask, g["hmask"])
    assert np.array_equal(da.etype, g["etype"])
    assert np.array_equal(da.node_xyz[da.nodes], g["elem_node_xyz"])


def test_matvec_matches_reference(oracle):
    g = np.load(os.path.join(GOLDEN, "ref_da.npz"))
    da = oracle.DA(g["bal"], 30)
    y = da.matvec(cases.nodal_function(da.node_xyz))
    ref = dict(zip(map(tuple, g["mv_xyz"]), g["mv_val"]))
    r = np.array([ref[tuple(v)] for v in da.node_xyz])
    assert np.linalg.norm(y - r) <= 1e-12 * np.linalg.norm(r)


def test_checkers_detect_defects(oracle, ref_cases):
    bal = ref_cases["gauss3k/bal"].copy()
    assert all(oracle.checks(bal, 30).values())
    # unsorted
    sw = bal.copy()
    sw[[5, 6]] = sw[[6, 5]]
    assert not oracle.checks(sw, 30)["sorted"]
    # incomplete: drop one octant
    assert not oracle.checks(np.delete(bal, 10, axis=0), 30)["complete"]
    # unbalanced: the unbalanced construction output of a clustered cloud
    assert not oracle.checks(ref_cases["clustered1k/lin"], 30)["balanced"]


def test_balance_idempotent_and_small_inputs(oracle, ref_cases):
    bal = ref_cases["gauss3k/bal"]
    assert np.array_equal(oracle.balance(bal, 30), bal)
    root = np.zeros((1, 4), np.uint32)
    assert np.array_equal(oracle.balance(root, 30), root)
    # the 8 children of the root
    kids = np.array([[(c & 1) << 29, (c >> 1 & 1) << 29, (c >> 2 & 1) << 29, 1] for c in range(8)], np.uint32)
    kids = kids[np.lexsort((kids[:, 0], kids[:, 1], kids[:, 2]))]
    assert np.array_equal(oracle.balance(kids, 30), kids)


# ---- balanceOctree(incCorner = false): faces and edges only ----------------
@pytest.fixture(scope="module")
def ref_face_edge():
    return np.load(os.path.join(GOLDEN, "ref_face_edge.npz"))


def _face_edge_names():
    g = np.load(os.path.join(GOLDEN, "ref_face_edge.npz"))
    return sorted({k.split("/")[0] for k in g.files})


@pytest.mark.parametrize("name", _face_edge_names())
def test_face_edge_balance_matches_reference(oracle, ref_face_edge, name):
    depth = int(ref_face_edge[f"{name}/params"][0])
    lin = ref_face_edge[f"{name}/lin"]
    bal = oracle.balance(lin, depth, inc_corner=False)
    assert len(bal) == int(ref_face_edge[f"{name}/bal_n"])
    assert oracle.fnv1a(bal) == int(ref_face_edge[f"{name}/bal_fnv"])
    ref = ref_face_edge[f"{name}/bal"]
    if len(ref):
        assert np.array_equal(bal, ref)
    chk = oracle.checks(bal, depth)
    assert chk["complete"] and chk["linear"] and chk["balanced_face_edge"]


# ---- SFC_treeSort -----------------------------------------------------------
def test_treesort_fixture_is_sort_and_linearise():
    """The reference's tree sort output (ref_treesort.npz) is the sorted input
    (option 0) and the sorted, unique input without ancestors
    (TS_REMOVE_DUPLICATES), except that a single input octant gives an empty
    pOutSorted (sfcSort.h:532 only fills it for two or more)."""
    g = np.load(os.path.join(GOLDEN, "ref_treesort.npz"))
    for name in sorted({k.split("/")[0] for k in g.files}):
        D = int(g[f"{name}/params"][0])
        inp, o0, o1 = g[f"{name}/in"], g[f"{name}/opt0"], g[f"{name}/opt1"]
        if len(inp) == 0:
            assert len(o0) == 0 and len(o1) == 0
            continue
        assert np.array_equal(np.unique(o0, axis=0), np.unique(inp, axis=0)) and len(o0) == len(inp)
        srt = cases.morton_sort(inp, D)
        assert np.array_equal(np.unique(o0, axis=0).shape, srt.shape)
        if len(inp) == 1:
            assert len(o1) == 0
            continue
        keep = np.ones(len(srt), bool)
        for i in range(len(srt) - 1):
            a, b = srt[i].astype(np.int64), srt[i + 1].astype(np.int64)
            if a[3] < b[3] and all((a[k] >> (D - a[3])) == (b[k] >> (D - a[3])) for k in range(3)):
                keep[i] = False
        assert np.array_equal(o1, srt[keep]), name
