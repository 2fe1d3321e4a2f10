"""Golden data at the benchmark workloads' own sizes, from the REFERENCE.

Runs the reference's own code (oracle/_ref/ref_driver, built from the
reference sources by oracle/Makefile) on the seeded workloads and writes
counts and SHA-256 digests of its outputs to tests/golden/ref_configs.json
(the arrays themselves are too large to keep):

  plain1m     1e6 N(0.5, 0.1^2) points (seed 0), maxDepth 30, maxPts 1:
              points2Octree and balanceOctree(incCorner = 1) outputs; the
              ot::DA element data (per element: level, child number,
              hanging mask, element type and the 8 node coordinates) and one
              FP64 Laplacian + mass matVec of config1_vector, summarised by
              its norm, 4 projections and 4096 sampled nodes
  lognormal64m 64e6 log-normal points (seed 0): points2Octree and
              balanceOctree outputs (balance through the 1-rank body with
              the raised ripple limit: the reference's own limit returns an
              empty octree above 1e7 octants)
  batch256    the 256 Gaussian-mixture clouds of the batching workload
              (datagen.batch_clouds): each cloud's points2Octree and
              balanceOctree outputs

Octant records are {x, y, z, level} uint32 little-endian in the reference's
Morton order; digests cover the record bytes.

Usage:  python tests/golden/make_golden_configs.py REFERENCE_DIR plain1m|lognormal64m|batch256 [--jobs N]
(REFERENCE_DIR may instead come from the DENDRO_REFERENCE environment variable.)
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dendro_gb300 import datagen  # noqa: E402
from tests.golden import cases  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
OUT = os.path.join(HERE, "ref_configs.json")
RIPPLE_LIMIT = 10_000_000  # the reference's default comboRipple limit (_COMBO_RIPPLE_FACTOR_)


def run(scratch, *args):
    args = [os.path.abspath(a) if isinstance(a, str) and os.sep in a else a for a in args]
    r = subprocess.run([DRIVER, *map(str, args)], capture_output=True, text=True, check=True, cwd=scratch)
    return json.loads(r.stdout.strip().splitlines()[-1])


def write_pts(path, p):
    with open(path, "wb") as f:
        f.write(np.uint64(len(p)).tobytes())
        f.write(np.ascontiguousarray(p, np.float64).tobytes())


def read_oct(path):
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(8), np.uint64)[0])
        return np.fromfile(f, np.uint32, 4 * n).reshape(n, 4)


def p2o_bal(scratch, name, pts, depth=30, maxpts=1):
    """Reference points2Octree then balanceOctree(incCorner = 1): counts,
    digests and seconds; the balanced records are returned too."""
    pf, of, bf = (os.path.join(scratch, f"{name}.{e}") for e in ("pts", "oct", "bal"))
    write_pts(pf, pts)
    i1 = run(scratch, "p2o", pf, depth, maxpts, of)
    os.remove(pf)
    lin = read_oct(of)
    patched = int(len(lin) > RIPPLE_LIMIT)
    i2 = run(scratch, "bal", of, depth, 1, patched, bf)
    os.remove(of)
    bal = read_oct(bf)
    os.remove(bf)
    rec = {"n_pts": len(pts), "sha_pts": cases.sha256_records(pts), "n_lin": len(lin),
           "sha_lin": cases.sha256_records(lin), "n_bal": len(bal), "sha_bal": cases.sha256_records(bal),
           "ref_seconds": {"p2o": i1["seconds"], "bal": i2["seconds"]}, "ripple_limit_raised": bool(patched)}
    return rec, bal


def plain1m(ref, scratch):
    pts = datagen.workload("gauss1m")
    rec, bal = p2o_bal(scratch, "plain1m", pts)
    bf = os.path.join(scratch, "plain1m.bal")
    with open(bf, "wb") as f:
        f.write(np.uint64(len(bal)).tobytes())
        f.write(bal.tobytes())
    prefix = os.path.join(scratch, "plain1m")
    stencils = os.path.join(ref, "Stencils")
    run(scratch, "da", bf, 30, stencils, "-", prefix)
    e = np.fromfile(prefix + ".elem", np.uint32, offset=8).reshape(-1, 28)
    node_xyz = np.unique(e[:, 4:].reshape(-1, 3), axis=0)
    order = cases.morton_rank_order(node_xyz)
    x = cases.config1_vector(node_xyz, 1, order)
    vrec = np.zeros(len(node_xyz), dtype=[("x", "<u4"), ("y", "<u4"), ("z", "<u4"), ("p", "<u4"), ("v", "<f8")])
    vrec["x"], vrec["y"], vrec["z"] = node_xyz.T
    vrec["v"] = x
    vf = os.path.join(scratch, "plain1m.vec")
    with open(vf, "wb") as f:
        f.write(np.uint64(len(vrec)).tobytes())
        f.write(vrec.tobytes())
    info = run(scratch, "da", bf, 30, stencils, vf, prefix)
    mv = np.fromfile(prefix + ".mv", dtype=vrec.dtype, offset=8)
    mv_xyz = np.stack([mv["x"], mv["y"], mv["z"]], 1)
    # y in the order of node_xyz (np.unique sorted it lexicographically)
    pos = np.lexsort(mv_xyz.T[::-1])
    assert np.array_equal(mv_xyz[pos], node_xyz)
    y = mv["v"][pos]
    w = np.stack([cases.config1_vector(node_xyz, 100 + j, order) for j in range(4)])
    sample = order[:: max(1, len(order) // 4096)][:4096]
    rec.update({
        "da": {"n_elem": int(len(e)), "n_node": int(info["n_nodes_da"]),
               "sha_elem": cases.sha256_records(e[:, 3:]),
               "elem_columns": "meta (DA level | child << 8 | hmask << 16 | etype << 24), then 8 x (x, y, z) "
                               "of the element's node (a hanging vertex: the parent's vertex)",
               "ref_seconds": {k: info[k] for k in info if k.startswith("t")}},
        "matvec_fp64": {"vector": "config1_vector(node_xyz, seed 1)", "norm2": float(np.linalg.norm(y)),
                        "max_abs": float(np.max(np.abs(y))), "projections": [float(v) for v in w @ y],
                        "projection_weights": "config1_vector(node_xyz, 100 + j), j = 0..3",
                        "sample_xyz": node_xyz[sample].tolist(), "sample_y": [float(v) for v in y[sample]]},
    })
    return rec


def lognormal64m(ref, scratch):
    pts = datagen.workload("lognormal64m")
    rec, _ = p2o_bal(scratch, "lognormal64m", pts)
    return rec


def batch256(ref, scratch, jobs):
    clouds = datagen.batch_clouds()
    out = [None] * len(clouds)

    def one(i):
        r, _ = p2o_bal(scratch, f"cloud{i}", clouds[i])
        return i, r

    order = sorted(range(len(clouds)), key=lambda i: -len(clouds[i]))  # largest first
    with cf.ThreadPoolExecutor(jobs) as ex:
        for i, r in ex.map(one, order):
            out[i] = r
            print(f"cloud {i}: {r['n_pts']} pts -> {r['n_bal']} balanced", flush=True)
    return {"clouds": out, "n_pts": int(sum(len(c) for c in clouds))}


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = os.environ.get("DENDRO_REFERENCE") if len(args) < 2 else args[0]
    which = args[-1] if args else None
    if not ref or not os.path.isdir(os.path.join(ref, "src")) or which not in ("plain1m", "lognormal64m", "batch256"):
        sys.exit(__doc__)
    jobs = int(next((a.split("=")[1] for a in sys.argv if a.startswith("--jobs=")), "6"))
    if not os.path.exists(DRIVER):
        subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), f"REF={ref}"])
    t0 = time.time()
    with tempfile.TemporaryDirectory(prefix="dendro_cfg_") as scratch:
        if which == "plain1m":
            rec = plain1m(ref, scratch)
        elif which == "lognormal64m":
            rec = lognormal64m(ref, scratch)
        else:
            rec = batch256(ref, scratch, jobs)
    rec["generated_seconds"] = time.time() - t0
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    data[which] = rec
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    print(f"{which}: written to {OUT} in {rec['generated_seconds']:.0f} s")


if __name__ == "__main__":
    main()
