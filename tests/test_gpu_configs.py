"""Parity at the benchmark workloads' own sizes, against the REFERENCE's own
outputs (tests/golden/ref_configs.json, written by
tests/golden/make_golden_configs.py from the reference binary):

  plain1m       1e6 N(0.5, 0.1^2) points: points2Octree and
                balanceOctree(incCorner = 1) bit-exact; the DA's per-element
                data bit-exact (level, child number, hanging mask, element
                type, the 8 node coordinates); the FP64 Laplacian + mass
                matVec within 1e-12 of the reference's on 4096 sampled nodes
                and 4 projections, FP32 within 1e-6 of FP64; the C
                restatement of the oracle bit-exact as well
  lognormal64m  64e6 log-normal points: build + balance bit-exact
  batch256      the 256 Gaussian-mixture clouds of the batching workload in
                one segmented build + balance: every cloud bit-exact

Digests are SHA-256 over the {x, y, z, level} uint32 records.  Each test
first checks that this platform regenerates the reference's input points bit
for bit (sha_pts)."""
import json
import os

import numpy as np
import pytest

from dendro_gb300 import DA, balanceOctree, datagen, points2Octree, points2OctreeBatch
from tests.golden import cases as gcases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FP64_RTOL = 1e-12
FP32_RTOL = 1e-6


def _ref(name):
    data = json.load(open(os.path.join(GOLDEN, "ref_configs.json")))
    if name not in data:
        pytest.skip(f"{name} not in ref_configs.json")
    return data[name]


sha = gcases.sha256_records


def _find_rows(table, rows):
    """Index in ``table`` of every row of ``rows`` (each present once)."""
    def h(a):
        a = a.astype(np.uint64)
        return (a[:, 0] * np.uint64(0x9E3779B97F4A7C15)) ^ (a[:, 1] * np.uint64(0xC2B2AE3D27D4EB4F)) ^ a[:, 2]

    cand = np.nonzero(np.isin(h(table), h(rows)))[0]
    where = {tuple(table[i]): i for i in cand}
    return np.array([where[tuple(r)] for r in rows])


@pytest.fixture(scope="module")
def plain1m(ctx):
    ref = _ref("plain1m")
    pts = datagen.workload("gauss1m")
    assert sha(pts) == ref["sha_pts"], "input points differ from the reference run's"
    lin = points2Octree(pts, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
    bal = balanceOctree(lin)
    return ref, pts, lin, bal


def test_plain1m_octree_bit_exact(plain1m):
    ref, _, lin, bal = plain1m
    a, b = lin.to_numpy(), bal.to_numpy()
    assert (len(a), sha(a)) == (ref["n_lin"], ref["sha_lin"])
    assert (len(b), sha(b)) == (ref["n_bal"], ref["sha_bal"])


def test_plain1m_c_restatement_bit_exact(plain1m):
    from oracle import dg_oracle

    ref, pts, lin, bal = plain1m
    o_lin = dg_oracle.points_to_octree(pts, 30, 1)
    assert sha(o_lin) == ref["sha_lin"]
    o_bal = dg_oracle.balance(o_lin, 30)
    assert sha(o_bal) == ref["sha_bal"]
    assert np.array_equal(o_bal, bal.to_numpy())


def test_plain1m_da_and_matvec(plain1m):
    ref, _, _, bal = plain1m
    rda, rmv = ref["da"], ref["matvec_fp64"]
    da = DA(bal)
    try:
        assert (da.n_elem, da.n_node) == (rda["n_elem"], rda["n_node"])
        d = da.download()
        rec = np.empty((da.n_elem, 25), np.uint32)
        rec[:, 0] = ((d["level"].astype(np.uint32) + 1) | (d["child"].astype(np.uint32) << 8)
                     | (d["hmask"].astype(np.uint32) << 16) | (d["etype"].astype(np.uint32) << 24))
        rec[:, 1:] = d["node_xyz"][d["nodes"]].reshape(da.n_elem, 24)
        assert sha(rec) == rda["sha_elem"], "DA element data differ from the reference's"
        xyz = d["node_xyz"]
        order = gcases.morton_rank_order(xyz)
        x = gcases.config1_vector(xyz, 1, order)
        y64 = da.matvec(x, precision=64)
        scale = rmv["max_abs"]
        assert abs(np.linalg.norm(y64) - rmv["norm2"]) <= FP64_RTOL * rmv["norm2"]
        w = np.stack([gcases.config1_vector(xyz, 100 + j, order) for j in range(4)])
        proj = w @ y64
        for p, q in zip(proj, rmv["projections"]):
            assert abs(p - q) <= FP64_RTOL * np.sqrt(da.n_node) * scale
        # the sampled nodes, looked up by coordinate
        sx = np.asarray(rmv["sample_xyz"], np.uint32)
        idx = _find_rows(xyz, sx)
        assert np.array_equal(xyz[idx], sx)
        err = np.max(np.abs(y64[idx] - np.asarray(rmv["sample_y"])))
        assert err <= FP64_RTOL * scale, err
        y32 = da.matvec(x.astype(np.float32), precision=32).astype(np.float64)
        assert np.linalg.norm(y32 - y64) <= FP32_RTOL * np.linalg.norm(y64)
    finally:
        da.free()


def test_lognormal64m_octree_bit_exact(ctx):
    ref = _ref("lognormal64m")
    pts = datagen.workload("lognormal64m")
    assert sha(pts) == ref["sha_pts"], "input points differ from the reference run's"
    lin = points2Octree(pts, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
    del pts
    a = lin.to_numpy()
    assert (len(a), sha(a)) == (ref["n_lin"], ref["sha_lin"])
    del a
    bal = balanceOctree(lin)
    lin.free()
    b = bal.to_numpy()
    bal.free()
    assert (len(b), sha(b)) == (ref["n_bal"], ref["sha_bal"])


def test_batch256_every_cloud_bit_exact(ctx):
    ref = _ref("batch256")["clouds"]
    clouds = datagen.batch_clouds()
    assert len(clouds) == len(ref)
    for i, c in enumerate(clouds):
        assert sha(c) == ref[i]["sha_pts"], f"cloud {i}: input points differ from the reference run's"
    lin = points2OctreeBatch(clouds, ctx=ctx)
    del clouds
    bal = balanceOctree(lin)
    off_l, off_b = lin.segments(), bal.segments()
    assert np.array_equal(np.diff(off_l), [r["n_lin"] for r in ref])
    assert np.array_equal(np.diff(off_b), [r["n_bal"] for r in ref])
    bad = []
    for name, oct_, off in (("lin", lin, off_l), ("bal", bal, off_b)):
        recs = oct_.to_numpy()
        for i, r in enumerate(ref):
            if sha(recs[off[i]:off[i + 1]]) != r[f"sha_{name}"]:
                bad.append((name, i))
        del recs
        oct_.free()
    assert not bad, f"clouds differing from the reference: {bad[:10]}"
