"""Generate the golden fixtures of tests/golden from the REFERENCE itself.

Runs the reference's own code (oracle/_ref/ref_driver, built from the
reference sources by oracle/Makefile) on seeded inputs and stores its
outputs next to the inputs:

  ref_cases.npz   points2Octree and balanceOctree outputs for small inputs
  ref_da.npz      ot::DA element data and one Laplacian+mass matVec
  ref_tables.npz  element-type masks (include/oda/cnumEtypes.h) and
                  statistics of the type-2 stencil tables and of the
                  restriction stencils RmatType1/2 (Stencils/*.inp)
  ref_hashes.json counts and FNV-1a hashes of larger octrees
  ref_complete.npz completeOctree outputs (cases.complete_inputs), or the
                  reference's abort on inputs that hold an octant and a
                  descendant in its first child (getNCA's assertion,
                  src/octFunctions.cpp:310)
  io/             the reference's point and octree files
  ref_mat.npz     the assembled K + M of CreateAndComputeFullJacobian1 on
                  a small balanced octree (row, column node coordinates)
  ref_face_edge.npz balanceOctree(incCorner = false) outputs
  ref_treesort.npz SFC::parSort::SFC_treeSort outputs (sort only, and
                  TS_REMOVE_DUPLICATES) on octant sets with repeats and
                  ancestors
  ref_mg_ops.npz  the reference's own operators on cases.TRANSFER:
                  restriction and prolongation (restrictMatVecType1 /
                  prolongMatVecType1 with the Dirichlet DOFs suppressed)
                  between a balanced octree and its next coarser level, the
                  Dirichlet operator and diagonal (DirichletJacobianMatMult /
                  DirichletJacobianMatGetDiagonal) on the finer one, and on
                  the level-0 octrees the element-loop MatShell callbacks
                  (Jacobian1MatMult / Jacobian1MatGetDiagonal, MassMatMult /
                  MassMatGetDiagonal, Jacobian2MatMult /
                  Jacobian2MatGetDiagonal with cases.element_factors)
  ref_assemble.npz the reference's assembled matrices on cases.ASSEMBLE
                  (CreateAndComputeFullJacobian1, ComputeDirichletJacobian and
                  ComputeJacobian2 with cases.element_factors, through
                  DA::setValuesInMatrix), as cases.csr_summary
  ref_hilbert.npz the reference's default Hilbert-ordered build
                  (oracle/_ref_hilbert/ref_driver, make ORDER=hilbert):
                  points2Octree, balanceOctree and completeOctree outputs

Usage:  python tests/golden/make_golden.py REFERENCE_DIR   (or DENDRO_REFERENCE=REFERENCE_DIR)
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import tempfile
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dendro_gb300 import datagen  # noqa: E402
from tests.golden import cases  # noqa: E402

REF = next((a for a in sys.argv[1:] if not a.startswith("--")), os.environ.get("DENDRO_REFERENCE"))
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    sys.exit("usage: make_golden.py REFERENCE_DIR (or set DENDRO_REFERENCE): the Dendro4 source tree")
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
DRIVER_HILBERT = os.path.join(ROOT, "oracle", "_ref_hilbert", "ref_driver")


SCRATCH = tempfile.mkdtemp(prefix="dendro_golden_")


def run(*args):
    # the reference's property checks write their failure dumps (.ot, .vtk)
    # into the working directory: run it in a scratch directory, with
    # absolute paths for every file argument
    args = [os.path.abspath(a) if isinstance(a, str) and os.sep in a else a for a in args]
    r = subprocess.run([DRIVER, *map(str, args)], capture_output=True, text=True, check=True, cwd=SCRATCH)
    return json.loads(r.stdout.strip().splitlines()[-1])


def write_pts(path, p):
    with open(path, "wb") as f:
        f.write(np.uint64(len(p)).tobytes())
        f.write(np.ascontiguousarray(p, np.float64).tobytes())


def read_oct(path):
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[:8], np.uint64)[0])
    return np.frombuffer(b[8:], np.uint32).reshape(n, 4).copy()


def write_oct(path, o):
    with open(path, "wb") as f:
        f.write(np.uint64(len(o)).tobytes())
        f.write(np.ascontiguousarray(o, np.uint32).tobytes())


def fnv1a(o):
    h = 1469598103934665603
    for byte in np.ascontiguousarray(o, np.uint32).tobytes():
        h ^= byte
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def ref_p2o_bal(tmp, name, pts, depth, maxpts):
    """Reference points2Octree then balanceOctree; the balanced octree is
    None when the reference aborts (it asserts on octants outside the domain,
    which its construction emits for some inputs with repeated points)."""
    pf, of, bf = (os.path.join(tmp, f"{name}.{e}") for e in ("pts", "oct", "bal"))
    write_pts(pf, pts)
    run("p2o", pf, depth, maxpts, of)
    lin = read_oct(of)
    try:
        run("bal", of, depth, 1, 1, bf)
    except subprocess.CalledProcessError:
        return lin, None
    return lin, read_oct(bf)


def make_io():
    """The reference's own writers (writePtsToFile, writeNodesToFile,
    writeNodesToFile_binary) on the balanced octree of a 200-point cloud, and
    what its readers return for those files: tests/golden/io/."""
    outdir = os.path.join(HERE, "io")
    os.makedirs(outdir, exist_ok=True)
    pts = datagen.gaussian(200, 0.5, 0.1, seed=11)
    with tempfile.TemporaryDirectory() as tmp:
        pf = os.path.join(tmp, "in.bin")
        write_pts(pf, pts)
        info = run("io", pf, 30, os.path.join(outdir, "gauss200"))
    np.save(os.path.join(outdir, "gauss200_points.npy"), pts)
    with open(os.path.join(outdir, "gauss200.json"), "w") as f:
        json.dump(info, f, indent=1, sort_keys=True)


def make_complete():
    """ot::completeOctree on cases.complete_inputs(): ref_complete.npz."""
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        fi, fo = os.path.join(tmp, "in.oct"), os.path.join(tmp, "out.oct")
        for name, octs, D, uniq, srt in cases.complete_inputs():
            write_oct(fi, octs)
            try:
                run("complete", fi, D, uniq, srt, fo)
                res, aborted = read_oct(fo), False
            except subprocess.CalledProcessError as e:
                assert "getNCA" in e.stderr, e.stderr
                res, aborted = np.zeros((0, 4), np.uint32), True
            out[f"{name}/in"] = octs
            out[f"{name}/params"] = np.array([D, uniq, srt], np.int64)
            out[f"{name}/out"] = res
            out[f"{name}/aborted"] = np.bool_(aborted)
    np.savez_compressed(os.path.join(HERE, "ref_complete.npz"), **out)


def run_hilbert(*args, timeout=20):
    """The Hilbert build; None when it aborts or does not finish in time
    (its construction walk runs for minutes or forever on some clustered
    inputs that the Morton build finishes in milliseconds)."""
    args = [os.path.abspath(a) if isinstance(a, str) and os.sep in a else a for a in args]
    try:
        r = subprocess.run([DRIVER_HILBERT, *map(str, args)], capture_output=True, text=True, cwd=SCRATCH,
                           timeout=timeout)
    except subprocess.TimeoutExpired:
        return None
    return None if r.returncode else json.loads(r.stdout.strip().splitlines()[-1])


def make_hilbert():
    """The Hilbert build on the small point cases (points2Octree then
    balanceOctree) and on the completeOctree inputs given in any order:
    ref_hilbert.npz."""
    if not os.path.exists(DRIVER_HILBERT):
        subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "ORDER=hilbert"])
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        pf, of, bf = (os.path.join(tmp, f"h.{e}") for e in ("pts", "oct", "bal"))
        for name, (fn, depth, maxpts) in cases.SMALL.items():
            write_pts(pf, fn())
            ok = run_hilbert("p2o", pf, depth, maxpts, of) is not None
            ok = ok and run_hilbert("bal", of, depth, 1, 0, bf) is not None
            out[f"p2o_{name}/finished"] = np.bool_(ok)
            for what, f in (("lin", of), ("bal", bf)):
                o = read_oct(f) if ok else np.zeros((0, 4), np.uint32)
                # large outputs as count + FNV-1a of the records in order
                out[f"p2o_{name}/{what}_n"] = np.int64(len(o))
                out[f"p2o_{name}/{what}_fnv"] = np.uint64(fnv1a(o))
                out[f"p2o_{name}/{what}"] = o if len(o) <= 4000 else np.zeros((0, 4), np.uint32)
            out[f"p2o_{name}/params"] = np.array([depth, maxpts], np.int64)
        fi, fo = os.path.join(tmp, "in.oct"), os.path.join(tmp, "out.oct")
        for name, octs, D, uniq, srt in cases.complete_inputs():
            if not name.endswith("_any") and name.startswith("sparse"):
                continue
            write_oct(fi, octs)
            ok = run_hilbert("complete", fi, D, 0, 0, fo) is not None
            out[f"complete_{name}/finished"] = np.bool_(ok)
            o = read_oct(fo) if ok else np.zeros((0, 4), np.uint32)
            out[f"complete_{name}/out_n"] = np.int64(len(o))
            out[f"complete_{name}/out_fnv"] = np.uint64(fnv1a(o))
            out[f"complete_{name}/out"] = o if len(o) <= 4000 else np.zeros((0, 4), np.uint32)
            out[f"complete_{name}/params"] = np.array([D], np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_hilbert.npz"), **out)


def make_mat():
    """The reference's assembled K + M (CreateAndComputeFullJacobian1,
    odaJac.C:470) on the balanced octree of cases.mat_points():
    ref_mat.npz with the entries as indices into the sorted node
    coordinates."""
    with tempfile.TemporaryDirectory() as tmp:
        _, bal = ref_p2o_bal(tmp, "mat", cases.mat_points(), 30, 1)
        bf = os.path.join(tmp, "mat.bal")
        write_oct(bf, bal)
        prefix = os.path.join(tmp, "mat")
        run("da", bf, 30, os.path.join(REF, "Stencils"), "-", prefix, "mat")
        b = open(prefix + ".mat", "rb").read()
        n = int(np.frombuffer(b[:8], np.uint64)[0])
        rec = np.frombuffer(b[8:], dtype=[("rc", "<u4", (6,)), ("v", "<f8")], count=n)
    rc = rec["rc"]
    node_xyz = np.unique(rc.reshape(-1, 3), axis=0)
    def index(xyz):
        pos = np.searchsorted(node_xyz.view([("", node_xyz.dtype)] * 3).ravel(),
                              np.ascontiguousarray(xyz).view([("", xyz.dtype)] * 3).ravel())
        return pos.astype(np.uint32)
    np.savez_compressed(os.path.join(HERE, "ref_mat.npz"), bal=bal, node_xyz=node_xyz,
                        row=index(rc[:, :3]), col=index(rc[:, 3:]), val=rec["v"].copy())


def read_vec(path):
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[:8], np.uint64)[0])
    rec = np.frombuffer(b[8:], dtype=[("c", "<u4", (4,)), ("v", "<f8")], count=n)
    return rec["c"][:, :3].copy(), rec["v"].copy()


def write_vec(path, xyz, v):
    rec = np.zeros(len(v), dtype=[("c", "<u4", (4,)), ("v", "<f8")])
    rec["c"][:, :3] = xyz
    rec["v"] = v
    with open(path, "wb") as f:
        f.write(np.uint64(len(v)).tobytes())
        f.write(rec.tobytes())


def write_coef(path, octs, coef):
    rec = np.zeros(len(octs), dtype=[("c", "<u4", (4,)), ("v", "<f8", (2,))])
    rec["c"], rec["v"] = octs, coef
    with open(path, "wb") as f:
        f.write(np.uint64(len(octs)).tobytes())
        f.write(rec.tobytes())


def make_mg_ops():
    """The reference's multigrid level operators (driver modes transfer and
    dirichlet) on cases.TRANSFER: per case the fine octree, the reference's
    coarse level, R v_f and P v_c, and A v_f and diag(A) of the Dirichlet
    operator on the fine level, by node coordinates, v =
    cases.hashed_nodal_values of the nodes.  The node coordinates of the
    inputs are the oracle's (test infrastructure), and the reference reports
    any node it did not find."""
    from oracle import dg_oracle

    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (fn, levels) in cases.TRANSFER.items():
            pf, of, bf = (os.path.join(tmp, f"{name}.{e}") for e in ("pts", "oct", "bal"))
            write_pts(pf, fn())
            run("p2o", pf, 30, 1, of)
            run("bal", of, 30, 1, 0, bf)
            fine = read_oct(bf)
            for _ in range(levels):
                cf = os.path.join(tmp, f"{name}.c")
                run("coarsen", bf, 30, cf)
                run("bal", cf, 30, 1, 0, bf)
                fine = read_oct(bf)
            coarse = dg_oracle.balance(dg_oracle.coarsen(fine, 30), 30)
            fxyz = dg_oracle.DA(fine, 30).node_xyz
            cxyz = dg_oracle.DA(coarse, 30).node_xyz
            vf, vc = os.path.join(tmp, f"{name}.vf"), os.path.join(tmp, f"{name}.vc")
            write_vec(vf, fxyz, cases.hashed_nodal_values(fxyz))
            write_vec(vc, cxyz, cases.hashed_nodal_values(cxyz))
            prefix = os.path.join(tmp, name)
            info = run("transfer", bf, 30, os.path.join(REF, "Stencils"), vf, vc, prefix)
            assert info["missing"] == 0 and info["conflicts"] == 0, info
            rx, rv = read_vec(prefix + ".r")
            px, pv = read_vec(prefix + ".p")
            info = run("dirichlet", bf, 30, os.path.join(REF, "Stencils"), vf, prefix)
            assert info["missing"] == 0 and info["conflicts"] == 0, info
            ax, av = read_vec(prefix + ".mv")
            dx, dv = read_vec(prefix + ".diag")
            assert np.array_equal(ax, dx)
            out[f"{name}/a_xyz"], out[f"{name}/a"], out[f"{name}/diag"] = ax, av, dv
            if levels == 0:
                cf = os.path.join(tmp, f"{name}.coef")
                write_coef(cf, fine, cases.element_factors(fine))
                info = run("jac", bf, 30, os.path.join(REF, "Stencils"), vf, cf, prefix)
                assert info["missing"] == 0 and info["conflicts"] == 0, info
                for op in ("j1", "j1d", "m", "md", "j2", "j2d"):
                    jx, out[f"{name}/{op}"] = read_vec(f"{prefix}.{op}")
                    assert np.array_equal(jx, ax)
            out[f"{name}/fine"] = fine
            out[f"{name}/coarse"] = read_oct(prefix + ".coarse")
            out[f"{name}/r_xyz"], out[f"{name}/r"] = rx, rv
            out[f"{name}/p_xyz"], out[f"{name}/p"] = px, pv
    np.savez_compressed(os.path.join(HERE, "ref_mg_ops.npz"), **out)


def read_mat(path):
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[:8], np.uint64)[0])
    rec = np.frombuffer(b[8:], dtype=[("rc", "<u4", (6,)), ("v", "<f8")], count=n)
    return rec["rc"].copy(), rec["v"].copy()


def make_assemble():
    """The reference's assembled matrices (driver mode assemble) on
    cases.ASSEMBLE: the node coordinates in lexicographic order and, per
    matrix, cases.csr_summary of its entries."""
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, fn in cases.ASSEMBLE.items():
            pf, of, bf, cf = (os.path.join(tmp, f"{name}.{e}") for e in ("pts", "oct", "bal", "coef"))
            write_pts(pf, fn())
            run("p2o", pf, 30, 1, of)
            run("bal", of, 30, 1, 0, bf)
            bal = read_oct(bf)
            write_coef(cf, bal, cases.element_factors(bal))
            prefix = os.path.join(tmp, name)
            info = run("assemble", bf, 30, os.path.join(REF, "Stencils"), cf, prefix)
            assert info["missing"] == 0 and info["conflicts"] == 0 and info["unmapped"] == 0, info
            mats = {m: read_mat(f"{prefix}.{m}") for m in ("k", "kd", "k2")}
            xyz = np.unique(np.concatenate([rc.reshape(-1, 3) for rc, _ in mats.values()]), axis=0)
            index = {tuple(p): i for i, p in enumerate(xyz.tolist())}
            out[f"{name}/bal"] = bal
            out[f"{name}/node_xyz"] = xyz
            for m, (rc, v) in mats.items():
                rows = np.array([index[tuple(p)] for p in rc[:, :3].tolist()])
                cols = np.array([index[tuple(p)] for p in rc[:, 3:].tolist()])
                for k, val in cases.csr_summary(xyz, rows, cols, v).items():
                    out[f"{name}/{m}/{k}"] = val
    np.savez_compressed(os.path.join(HERE, "ref_assemble.npz"), **out)


def make_face_edge():
    """balanceOctree with incCorner = false (faces and edges only) on the
    reference's points2Octree output of every small case whose balance
    finishes: ref_face_edge.npz (count + FNV-1a, and the records up to 50k
    octants)."""
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (fn, depth, maxpts) in cases.SMALL.items():
            pf, of, bf = (os.path.join(tmp, f"{name}.{e}") for e in ("pts", "oct", "bal"))
            write_pts(pf, fn())
            run("p2o", pf, depth, maxpts, of)
            try:
                run("bal", of, depth, 0, 0, bf)
            except subprocess.CalledProcessError:
                continue  # octants outside the domain: the reference's balance aborts
            lin, bal = read_oct(of), read_oct(bf)
            out[f"{name}/lin"] = lin
            out[f"{name}/bal_n"] = np.int64(len(bal))
            out[f"{name}/bal_fnv"] = np.uint64(fnv1a(bal))
            out[f"{name}/bal"] = bal if len(bal) <= 50000 else np.zeros((0, 4), np.uint32)
            out[f"{name}/params"] = np.array([depth, maxpts], np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_face_edge.npz"), **out)


def make_treesort():
    """SFC::parSort::SFC_treeSort at one rank (options 0: the input sorted in
    place; TS_REMOVE_DUPLICATES: sorted without repeats and ancestors) on the
    completeOctree inputs and on a shuffled, repeated balanced octree with
    ancestors: ref_treesort.npz."""
    rng = np.random.Generator(np.random.PCG64(77))
    inputs = [(name, octs, D) for name, octs, D, _, _ in cases.complete_inputs()]
    with tempfile.TemporaryDirectory() as tmp:
        _, bal = ref_p2o_bal(tmp, "ts", datagen.gaussian(1500, 0.5, 0.1, seed=78), 30, 1)
    anc = bal[rng.integers(0, len(bal), 200)].astype(np.int64)
    la = np.maximum(anc[:, 3] - rng.integers(1, 4, len(anc)), 0)
    m = ~((np.int64(1) << (30 - la)) - 1)
    anc = np.stack([anc[:, 0] & m, anc[:, 1] & m, anc[:, 2] & m, la], 1).astype(np.uint32)
    messy = np.concatenate([bal, bal[rng.integers(0, len(bal), 3000)], anc])
    rng.shuffle(messy)
    inputs.append(("bal1500_messy", messy, 30))
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        fi, fo = os.path.join(tmp, "in.oct"), os.path.join(tmp, "out.oct")
        for name, octs, D in inputs:
            write_oct(fi, octs)
            out[f"{name}/in"] = octs
            out[f"{name}/params"] = np.array([D], np.int64)
            for opt in (0, 1):
                run("treesort", fi, D, opt, fo)
                out[f"{name}/opt{opt}"] = read_oct(fo)
    np.savez_compressed(os.path.join(HERE, "ref_treesort.npz"), **out)


def main():
    if "--face-edge-only" in sys.argv:
        make_face_edge()
        return
    if "--treesort-only" in sys.argv:
        make_treesort()
        return
    if "--mat-only" in sys.argv:
        make_mat()
        return
    if "--mg-ops-only" in sys.argv:
        make_mg_ops()
        return
    if "--assemble-only" in sys.argv:
        make_assemble()
        return
    if "--hilbert-only" in sys.argv:
        make_hilbert()
        return
    if "--complete-only" in sys.argv:
        if not os.path.exists(DRIVER):
            subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}"])
        make_complete()
        return
    if "--io-only" in sys.argv:
        if not os.path.exists(DRIVER):
            subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}"])
        make_io()
        return
    if not os.path.exists(DRIVER):
        subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}"])
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (fn, depth, maxpts) in cases.SMALL.items():
            pts = fn()
            lin, bal = ref_p2o_bal(tmp, name, pts, depth, maxpts)
            out[f"{name}/pts"] = pts
            out[f"{name}/lin"] = lin
            out[f"{name}/bal_aborted"] = np.bool_(bal is None)
            if bal is None:
                bal = np.zeros((0, 4), np.uint32)
            # large balanced outputs are kept as count + FNV-1a only
            out[f"{name}/bal_n"] = np.int64(len(bal))
            out[f"{name}/bal_fnv"] = np.uint64(fnv1a(bal))
            out[f"{name}/bal"] = bal if len(bal) <= 50000 else np.zeros((0, 4), np.uint32)
            out[f"{name}/params"] = np.array([depth, maxpts], np.int64)
        np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **out)

        # DA + matVec on a small balanced octree
        pts = cases.da_points()
        _, bal = ref_p2o_bal(tmp, "da", pts, 30, 1)
        bf = os.path.join(tmp, "da.bal")
        write_oct(bf, bal)
        # nodes of the DA are only known after the DA is built: first pass
        # without a vector gives the element dump (node coordinates)
        prefix = os.path.join(tmp, "da")
        run("da", bf, 30, os.path.join(REF, "Stencils"), "-", prefix)
        e = open(prefix + ".elem", "rb").read()
        ne = int(np.frombuffer(e[:8], np.uint64)[0])
        E = np.frombuffer(e[8:], np.uint32).reshape(ne, 28)
        node_xyz = np.unique(E[:, 4:].reshape(-1, 3), axis=0)
        vals = cases.nodal_function(node_xyz)
        rec = np.zeros(len(node_xyz), dtype=[("x", "<u4"), ("y", "<u4"), ("z", "<u4"), ("p", "<u4"), ("v", "<f8")])
        rec["x"], rec["y"], rec["z"] = node_xyz.T
        rec["v"] = vals
        vf = os.path.join(tmp, "vec.bin")
        with open(vf, "wb") as f:
            f.write(np.uint64(len(rec)).tobytes())
            f.write(rec.tobytes())
        info = run("da", bf, 30, os.path.join(REF, "Stencils"), vf, prefix)
        m = open(prefix + ".mv", "rb").read()
        R = np.frombuffer(m[8:], dtype=rec.dtype)
        meta = E[:, 3]
        np.savez_compressed(
            os.path.join(HERE, "ref_da.npz"),
            bal=bal,
            level=(meta & 255).astype(np.uint8),
            child=((meta >> 8) & 255).astype(np.uint8),
            hmask=((meta >> 16) & 255).astype(np.uint8),
            etype=(meta >> 24).astype(np.uint8),
            elem_node_xyz=E[:, 4:].reshape(ne, 8, 3),
            mv_xyz=np.stack([R["x"], R["y"], R["z"]], 1),
            mv_val=R["v"].copy(),
            n_nodes=np.int64(info["n_nodes_da"]),
        )

        # larger cases: hashes only
        hashes = {}
        for name, (fn, depth, maxpts) in cases.LARGE.items():
            lin, bal = ref_p2o_bal(tmp, name, fn(), depth, maxpts)
            hashes[name] = {"n_lin": len(lin), "fnv_lin": f"{fnv1a(lin):016x}", "n_bal": len(bal),
                            "fnv_bal": f"{fnv1a(bal):016x}"}
        with open(os.path.join(HERE, "ref_hashes.json"), "w") as f:
            json.dump(hashes, f, indent=1, sort_keys=True)

    # tables
    src = open(os.path.join(REF, "include", "oda", "cnumEtypes.h")).read()
    blocks = re.split(r"class cNumEtype<(\d)>", src)[1:]
    order = ["ET_N", "ET_Y", "ET_X", "ET_XY", "ET_Z", "ET_ZY", "ET_ZX", "ET_ZXY", "ET_XY_XY", "ET_XY_ZXY", "ET_YZ_ZY",
             "ET_YZ_ZXY", "ET_YZ_XY_ZXY", "ET_ZX_ZX", "ET_ZX_ZXY", "ET_ZX_XY_ZXY", "ET_ZX_YZ_ZXY", "ET_ZX_YZ_XY_ZXY"]
    masks = np.zeros((8, 18), np.uint8)
    for i in range(0, len(blocks), 2):
        c = int(blocks[i])
        d = dict(re.findall(r"(ET_\w+)\s*=\s*(\d+)", blocks[i + 1]))
        masks[c] = [int(d[k]) for k in order]

    def stats(fname):
        a = np.array(open(os.path.join(REF, "Stencils", fname)).read().split(), np.float64).reshape(8, 18, 8, 8)
        w = np.arange(1, 65, dtype=np.float64).reshape(8, 8)
        return np.stack([a.sum((2, 3)), (a * a).sum((2, 3)), (a * w).sum((2, 3)), a[:, :, 0, :].sum(2)], -1)

    def rmat(fname, shape):
        a = np.array(open(os.path.join(REF, "Stencils", fname)).read().split(), np.float64)
        a = a[: int(np.prod(shape))].reshape(shape)
        w = np.arange(1, 65, dtype=np.float64).reshape(8, 8)
        return np.stack([a.sum((-2, -1)), (a * w).sum((-2, -1)), (a * a).sum((-2, -1))], -1)

    np.savez_compressed(os.path.join(HERE, "ref_tables.npz"), etype_masks=masks, lap_stats=stats("LapType2Stencils.inp"),
                        mass_stats=stats("MassType2Stencils.inp"),
                        rmat1_stats=rmat("RmatType1Stencils.inp", (8, 8, 18, 8, 8)),
                        rmat2_stats=rmat("RmatType2Stencils.inp", (8, 18, 8, 8)))
    print("golden fixtures written to", HERE)
    make_io()
    make_complete()
    make_hilbert()
    make_mat()
    make_mg_ops()
    make_assemble()
    make_face_edge()
    make_treesort()


if __name__ == "__main__":
    main()
