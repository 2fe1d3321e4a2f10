"""Parity of the CUDA path (through the C ABI) with the oracle.

Octrees must be bit-exact; the FP64 matVec within 1e-12 relative (L2) of
the oracle's FP64 element loop, the FP32 matVec within 1e-6 relative of it.
"""
import numpy as np
import pytest

from dendro_gb300 import DA, DendroError, Octree, balanceOctree, datagen, points2Octree, sortUniquePoints

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12
FP32_RTOL = 1e-6


def clustered(n, seed):
    """Points packed into a few tiny boxes: leaves down to maxDepth."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0.2, 0.8, size=(4, 3))
    p = c[rng.integers(0, 4, n)] + rng.uniform(0, 2.0 ** -27, size=(n, 3))
    return p


def boundary(n, seed):
    """Points on and next to the faces, edges and corners of the unit cube."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = rng.uniform(0, 1, size=(n, 3))
    hi = np.nextafter(1.0, 0.0)
    for a in range(3):
        sel = rng.random(n) < 0.3
        p[sel, a] = rng.choice([0.0, hi, 0.5, 2.0 ** -30, 1 - 2.0 ** -30], size=sel.sum())
    return p


CASES = {
    "gauss": lambda: datagen.gaussian(20000, 0.5, 0.1, seed=5),
    "lognormal": lambda: datagen.lognormal(20000, seed=6),
    "mixture": lambda: datagen.mixture(15000, np.random.Generator(np.random.PCG64(7))),
    "clustered": lambda: clustered(3000, 8),
    "boundary": lambda: boundary(4000, 9),
    "one": lambda: np.array([[0.3, 0.6, 0.9]]),
    "two": lambda: np.array([[0.1, 0.1, 0.1], [0.1 + 2.0 ** -30, 0.1, 0.1]]),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("max_pts", [1, 3])
def test_points2octree_bit_exact(ctx, oracle, case, max_pts):
    pts = CASES[case]()
    try:
        ref = oracle.points_to_octree(pts, 30, max_pts)
    except oracle.NoTermination:
        # heavily repeated points: the reference walk never ends; refused
        with pytest.raises(DendroError) as e:
            points2Octree(pts, maxDepth=30, maxNumPtsPerOctant=max_pts, ctx=ctx)
        assert e.value.status == 1
        return
    got = points2Octree(pts, maxDepth=30, maxNumPtsPerOctant=max_pts, ctx=ctx).to_numpy()
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("max_depth", [30, 12, 6])
def test_points2octree_depths(ctx, oracle, max_depth):
    pts = datagen.gaussian(5000, 0.5, 0.2, seed=11)
    ref = oracle.points_to_octree(pts, max_depth, 1)
    got = points2Octree(pts, maxDepth=max_depth, maxNumPtsPerOctant=1, ctx=ctx).to_numpy()
    assert np.array_equal(got, ref)


def test_points2octree_nonterminating_reference_walk(ctx, oracle):
    # 5000 points on a 16^3 grid repeat heavily; the reference walk then
    # climbs above the root and never terminates (it runs out of memory)
    pts = datagen.gaussian(5000, 0.5, 0.2, seed=11)
    with pytest.raises(oracle.NoTermination):
        oracle.points_to_octree(pts, 4, 1)
    with pytest.raises(DendroError) as e:
        points2Octree(pts, maxDepth=4, maxNumPtsPerOctant=1, ctx=ctx)
    assert e.value.status == 1


def test_points2octree_duplicates_follow_reference_walk(ctx, oracle):
    # repeated points make the reference walk skip refinements; the CUDA
    # path detects them and runs the walk verbatim
    base = datagen.gaussian(3000, 0.5, 0.1, seed=12)
    pts = np.concatenate([base, base[::7], base[::13]])
    ref = oracle.points_to_octree(pts, 30, 1)
    got = points2Octree(pts, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx).to_numpy()
    assert np.array_equal(got, ref)


def test_sort_unique_points(ctx, oracle):
    base = datagen.lognormal(30000, seed=13)
    pts = np.concatenate([base, base[:500]])
    ref = oracle.quantize_sort(pts, 30)
    keep = np.ones(len(ref), bool)
    keep[1:] = np.any(ref[1:] != ref[:-1], axis=1)
    got = sortUniquePoints(pts, maxDepth=30, ctx=ctx)
    assert np.array_equal(got, ref[keep])


def test_domain_error(ctx):
    with pytest.raises(DendroError) as e:
        points2Octree(np.array([[0.5, 0.5, 1.0], [0.1, 0.2, 0.3]]), ctx=ctx)
    assert e.value.status == 4
    with pytest.raises(DendroError):
        points2Octree(np.array([[np.nan, 0.5, 0.5], [0.1, 0.2, 0.3]]), ctx=ctx)


@pytest.mark.parametrize("case", ["gauss", "lognormal", "mixture", "clustered", "boundary", "one", "two"])
def test_balance_bit_exact(ctx, oracle, case):
    pts = CASES[case]()
    if case == "clustered":
        pts = np.unique(oracle.quantize_sort(pts, 30)[:, :3], axis=0).astype(np.float64) / (1 << 30)
    lin = oracle.points_to_octree(pts, 30, 1)
    if (lin[:, :3] >= (1 << 30)).any():
        # repeated points drove the construction walk outside the domain;
        # the reference asserts on such an octree, the CUDA path rejects it
        with pytest.raises(DendroError) as e:
            balanceOctree(Octree.from_numpy(lin, 30, ctx=ctx))
        assert e.value.status == 4
        return
    ref = oracle.balance(lin, 30)
    got = balanceOctree(Octree.from_numpy(lin, 30, ctx=ctx)).to_numpy()
    assert np.array_equal(got, ref)
    assert all(oracle.checks(got, 30).values())


def test_pipeline_resident(ctx, oracle):
    pts = datagen.gaussian(50000, 0.5, 0.1, seed=14)
    lin = points2Octree(pts, ctx=ctx)
    bal = balanceOctree(lin)
    ref = oracle.balance(oracle.points_to_octree(pts, 30, 1), 30)
    assert np.array_equal(bal.to_numpy(), ref)


def _da_parity(ctx, oracle, bal):
    oda = oracle.DA(bal, 30)
    da = DA(Octree.from_numpy(bal, 30, ctx=ctx))
    assert da.n_elem == oda.n_elem
    assert da.n_node == oda.n_node
    d = da.download()
    assert np.array_equal(d["level"], oda.level)
    assert np.array_equal(d["child"], oda.child)
    assert np.array_equal(d["hmask"], oda.hmask)
    assert np.array_equal(d["etype"], oda.etype)
    # element -> node maps agree by node coordinates
    assert np.array_equal(d["node_xyz"][d["nodes"]], oda.node_xyz[oda.nodes])
    return da, oda, d


def _to_oracle_order(d, oda):
    """permutation p with gpu_node[p[i]] == oracle node i (by coordinates)"""
    og = np.lexsort(d["node_xyz"].T[::-1])
    oo = np.lexsort(oda.node_xyz.T[::-1])
    assert np.array_equal(d["node_xyz"][og], oda.node_xyz[oo])
    p = np.empty(len(oo), np.int64)
    p[oo] = og
    assert np.array_equal(d["node_xyz"][p], oda.node_xyz)
    return p


@pytest.mark.parametrize("case", ["gauss", "lognormal", "clustered", "boundary", "one"])
def test_da_and_matvec(ctx, oracle, case):
    pts = CASES[case]()
    if case in ("boundary", "clustered"):
        pts = np.unique(oracle.quantize_sort(pts, 30)[:, :3], axis=0).astype(np.float64) / (1 << 30)
    lin = oracle.points_to_octree(pts, 30, 1)
    assert not (lin[:, :3] >= (1 << 30)).any()
    bal = oracle.balance(lin, 30)
    da, oda, d = _da_parity(ctx, oracle, bal)
    p = _to_oracle_order(d, oda)
    rng = np.random.Generator(np.random.PCG64(1))
    x_o = rng.uniform(-1.0, 1.0, oda.n_node)
    y_o = oda.matvec(x_o, 1.0, 1.0)
    x_g = np.empty(da.n_node)
    x_g[p] = x_o
    y64 = da.matvec(x_g, precision=64)[p]
    assert np.linalg.norm(y64 - y_o) <= FP64_RTOL * np.linalg.norm(y_o)
    y32 = da.matvec(x_g.astype(np.float32), precision=32)[p].astype(np.float64)
    assert np.linalg.norm(y32 - y_o) <= FP32_RTOL * np.linalg.norm(y_o)
    # material factors (-lapMatPropFac / -massMatPropFac)
    y_f = oda.matvec(x_o, 2.5, 0.25)
    yg_f = da.matvec(x_g, precision=64, lapFac=2.5, massFac=0.25)[p]
    assert np.linalg.norm(yg_f - y_f) <= FP64_RTOL * np.linalg.norm(y_f)


def test_da_rejects_unbalanced(ctx, oracle):
    pts = datagen.gaussian(2000, 0.5, 0.1, seed=15)
    lin = oracle.points_to_octree(pts, 30, 1)
    if oracle.checks(lin, 30)["balanced"]:
        pytest.skip("input happens to be balanced")
    with pytest.raises(DendroError) as e:
        DA(Octree.from_numpy(lin, 30, ctx=ctx))
    assert e.value.status == 5


# ---- against the reference's own outputs (tests/golden) -------------------
import json  # noqa: E402
import os  # noqa: E402

from tests.golden import cases as gcases  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fnv1a(o):
    h = 1469598103934665603
    for byte in np.ascontiguousarray(o, np.uint32).tobytes():
        h ^= byte
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


@pytest.mark.parametrize("name", sorted(gcases.SMALL))
def test_golden_reference_cases(ctx, name):
    g = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    depth, maxpts = (int(v) for v in g[f"{name}/params"])
    lin = points2Octree(g[f"{name}/pts"], maxDepth=depth, maxNumPtsPerOctant=maxpts, ctx=ctx)
    assert np.array_equal(lin.to_numpy(), g[f"{name}/lin"])
    if bool(g[f"{name}/bal_aborted"]):
        # the reference asserts on its own construction output here
        with pytest.raises(DendroError) as e:
            balanceOctree(lin)
        assert e.value.status == 4
        return
    bal = balanceOctree(lin).to_numpy()
    assert len(bal) == int(g[f"{name}/bal_n"])
    assert _fnv1a(bal) == int(g[f"{name}/bal_fnv"])


@pytest.mark.parametrize("name", sorted(gcases.LARGE))
def test_golden_reference_hashes(ctx, name):
    exp = json.load(open(os.path.join(GOLDEN, "ref_hashes.json")))[name]
    fn, depth, maxpts = gcases.LARGE[name]
    lin = points2Octree(fn(), maxDepth=depth, maxNumPtsPerOctant=maxpts, ctx=ctx)
    bal = balanceOctree(lin)
    a, b = lin.to_numpy(), bal.to_numpy()
    assert (len(a), f"{_fnv1a(a):016x}") == (exp["n_lin"], exp["fnv_lin"])
    assert (len(b), f"{_fnv1a(b):016x}") == (exp["n_bal"], exp["fnv_bal"])


def test_golden_reference_da_and_matvec(ctx):
    g = np.load(os.path.join(GOLDEN, "ref_da.npz"))
    da = DA(Octree.from_numpy(g["bal"], 30, ctx=ctx))
    assert (da.n_elem, da.n_node) == (len(g["bal"]), int(g["n_nodes"]))
    d = da.download()
    assert np.array_equal(d["level"] + 1, g["level"])
    assert np.array_equal(d["child"], g["child"])
    assert np.array_equal(d["hmask"], g["hmask"])
    assert np.array_equal(d["etype"], g["etype"])
    assert np.array_equal(d["node_xyz"][d["nodes"]], g["elem_node_xyz"])
    ref = dict(zip(map(tuple, g["mv_xyz"]), g["mv_val"]))
    r = np.array([ref[tuple(v)] for v in d["node_xyz"]])
    x = gcases.nodal_function(d["node_xyz"])
    y64 = da.matvec(x, precision=64)
    assert np.linalg.norm(y64 - r) <= FP64_RTOL * np.linalg.norm(r)
    y32 = da.matvec(x.astype(np.float32), precision=32).astype(np.float64)
    assert np.linalg.norm(y32 - r) <= FP32_RTOL * np.linalg.norm(r)


@pytest.mark.parametrize("name", ["gauss", "lognormal", "mixture"])
def test_fp32_matvec_both_loop_forms(ctx, oracle, name):
    """The FP32 element loop's run form (the default) and its pair form give
    the same operator: each within FP32_RTOL of the oracle's FP64 loop, and
    the Dirichlet level operator of a hierarchy likewise."""
    from dendro_gb300 import Context, MultiGrid

    pts = CASES[name]()
    c = Context(0)
    bal = balanceOctree(points2Octree(pts, ctx=c))
    da = DA(bal)
    d = da.download()
    oda = oracle.DA(bal.to_numpy(), 30)
    # a rough field (uniform in [-1, 1]): a smooth one cancels in the
    # Laplacian, and FP32 rounding then exceeds 1e-6 of the result in either form
    x = np.random.Generator(np.random.PCG64(9)).uniform(-1.0, 1.0, da.n_node)
    order_g = np.lexsort(d["node_xyz"].T[::-1])
    order_o = np.lexsort(oda.node_xyz.T[::-1])
    xo = np.empty(oda.n_node)
    xo[order_o] = x[order_g]
    ref = oda.matvec(xo)[order_o]
    ys = {}
    for form in ("runs", "pairs"):
        c.set_matvec_form(form)
        y = da.matvec(x.astype(np.float32), precision=32).astype(np.float64)[order_g]
        assert np.linalg.norm(y - ref) <= FP32_RTOL * np.linalg.norm(ref), form
        ys[form] = y
    assert np.linalg.norm(ys["runs"] - ys["pairs"]) <= FP32_RTOL * np.linalg.norm(ref)
    mg = MultiGrid(bal, max_coarse_elems=1000, ctx=c)
    z = {}
    for form in ("runs", "pairs"):
        c.set_matvec_form(form)
        z[form] = mg.matvec(0, x.astype(np.float32), precision=32).astype(np.float64)
    y64 = mg.matvec(0, x, precision=64)
    for form in ("runs", "pairs"):
        assert np.linalg.norm(z[form] - y64) <= FP32_RTOL * np.linalg.norm(y64), form
    c.set_matvec_form("runs")


@pytest.mark.parametrize("name", ["gauss", "mixture"])
def test_fp64_matvec_both_loop_forms(ctx, oracle, name):
    """The FP64 element loop in run form (the default) and in pair form:
    each within FP64_RTOL of the oracle's loop, and the Dirichlet level
    operator likewise between the two forms."""
    from dendro_gb300 import Context, MultiGrid

    pts = CASES[name]()
    c = Context(0)
    bal = balanceOctree(points2Octree(pts, ctx=c))
    da = DA(bal)
    d = da.download()
    oda = oracle.DA(bal.to_numpy(), 30)
    x = np.random.Generator(np.random.PCG64(11)).uniform(-1.0, 1.0, da.n_node)
    order_g = np.lexsort(d["node_xyz"].T[::-1])
    order_o = np.lexsort(oda.node_xyz.T[::-1])
    xo = np.empty(oda.n_node)
    xo[order_o] = x[order_g]
    ref = oda.matvec(xo)[order_o]
    ys = {}
    for form in ("runs", "pairs"):
        c.set_matvec_form(form)
        ys[form] = da.matvec(x, precision=64)[order_g]
        assert np.linalg.norm(ys[form] - ref) <= FP64_RTOL * np.linalg.norm(ref), form
    mg = MultiGrid(bal, max_coarse_elems=1000, ctx=c)
    z = {}
    for form in ("runs", "pairs"):
        c.set_matvec_form(form)
        z[form] = mg.matvec(0, x, precision=64)
    assert np.linalg.norm(z["runs"] - z["pairs"]) <= FP64_RTOL * np.linalg.norm(z["pairs"])
    c.set_matvec_form("runs")
