"""The rest of the reference's API on the path, through the C ABI and the C++
mirror, against the reference's own outputs and the oracle:

  * balanceOctree(incCorner = false), faces and edges only
    (tests/golden/ref_face_edge.npz, the oracle on larger clouds, and every
    cloud of a batch);
  * SFC::parSort::SFC_treeSort, sort only and TS_REMOVE_DUPLICATES
    (tests/golden/ref_treesort.npz);
  * a C++ caller written against the reference's surface (MPI_Comm
    parameters, ot::DA element loop and vectors, PETSc MatShell callbacks,
    SFC_treeSort, the omg hierarchy), tests/cpp/reference_surface_main.cpp.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from dendro_gb300 import (DA, Octree, balanceOctree, datagen, points2Octree, points2OctreeBatch, treeSort)
from dendro_gb300 import build as cuda_build

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _fnv(o):
    from oracle import dg_oracle

    return dg_oracle.fnv1a(o)


def test_face_edge_balance_matches_reference(ctx):
    g = np.load(os.path.join(GOLDEN, "ref_face_edge.npz"))
    names = sorted({k.split("/")[0] for k in g.files})
    assert len(names) >= 8
    for name in names:
        depth = int(g[f"{name}/params"][0])
        lin = Octree.from_numpy(g[f"{name}/lin"], depth, ctx=ctx)
        bal = balanceOctree(lin, incCorner=False).to_numpy()
        assert len(bal) == int(g[f"{name}/bal_n"]), name
        assert _fnv(bal) == int(g[f"{name}/bal_fnv"]), name
        if len(g[f"{name}/bal"]):
            assert np.array_equal(bal, g[f"{name}/bal"]), name


@pytest.mark.parametrize("maker", [
    lambda: datagen.lognormal(200_000, seed=61),
    lambda: datagen.mixture(150_000, np.random.Generator(np.random.PCG64(62))),
    lambda: datagen.gaussian(100_000, 0.5, 0.2, seed=63),
])
def test_face_edge_balance_matches_oracle(ctx, oracle, maker):
    pts = maker()
    lin = points2Octree(pts, ctx=ctx)
    bal = balanceOctree(lin, incCorner=False).to_numpy()
    ref = oracle.balance(lin.to_numpy(), 30, inc_corner=False)
    assert np.array_equal(bal, ref)
    full = balanceOctree(lin, incCorner=True).to_numpy()
    assert len(full) > len(bal)
    chk = oracle.checks(bal, 30)
    assert chk["balanced_face_edge"] and not chk["balanced"]


def test_face_edge_balance_batch_every_cloud(ctx, oracle):
    rng = np.random.Generator(np.random.PCG64(64))
    clouds = [datagen.mixture(int(n), rng) for n in rng.integers(1, 40_000, 12)]
    lin = points2OctreeBatch(clouds, ctx=ctx)
    bal = balanceOctree(lin, incCorner=False)
    for lo, bo in zip(lin.split(), bal.split()):
        assert np.array_equal(bo, oracle.balance(lo, 30, inc_corner=False))


def test_tree_sort_matches_reference(ctx):
    g = np.load(os.path.join(GOLDEN, "ref_treesort.npz"))
    names = sorted({k.split("/")[0] for k in g.files})
    for name in names:
        D = int(g[f"{name}/params"][0])
        inp = g[f"{name}/in"]
        o0 = treeSort(inp, maxDepth=D, options=0, ctx=ctx)
        assert np.array_equal(o0, g[f"{name}/opt0"]), name
        o1 = treeSort(inp, maxDepth=D, options=1, ctx=ctx)
        if len(inp) == 1:
            # the reference leaves pOutSorted empty below two octants; the
            # library returns the octant
            assert len(g[f"{name}/opt1"]) == 0 and np.array_equal(o1, inp)
        else:
            assert np.array_equal(o1, g[f"{name}/opt1"]), name
    from dendro_gb300 import DendroError

    with pytest.raises(DendroError):
        treeSort(g["root/in"], maxDepth=8, options=2, ctx=ctx)


def _compile(name, tmp_path, extra):
    lib = cuda_build.build()
    exe = tmp_path / name
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), *extra,
                           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-o", str(exe), lib,
                           "-Wl,-rpath," + os.path.dirname(lib)])
    return exe


def _read(path):
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[:8], np.uint64)[0])
    return np.frombuffer(b[8:], np.uint32).reshape(n, -1)


def test_reference_surface_caller(oracle, tmp_path):
    exe = _compile("reference_surface_main", tmp_path, ["-I", os.path.join(ROOT, "oracle", "ref_shim")])
    pts = datagen.gaussian(15_000, 0.5, 0.1, seed=65)
    pf = tmp_path / "p.pts"
    with open(pf, "wb") as f:
        f.write(np.uint64(len(pts)).tobytes())
        f.write(pts.tobytes())
    pre = str(tmp_path / "out")
    r = subprocess.run([str(exe), str(pf), pre], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    info = json.loads(r.stdout.strip().splitlines()[-1])
    lin = oracle.points_to_octree(pts, 30, 1)
    bal = oracle.balance(lin, 30)
    assert np.array_equal(_read(pre + ".bal"), bal)
    assert np.array_equal(_read(pre + ".bal18"), oracle.balance(lin, 30, inc_corner=False))
    assert info["active"] == 1 and info["petsc_rc"] == 0
    # the element loop visits every element once; the DA embeds one level deeper
    assert info["n_elem_loop"] == len(bal) and info["dependent_elems"] == 0 and info["maxD"] == 31
    assert info["volume"] == 1.0
    assert info["node_refs"] == 8 * len(bal)
    # per-element data from the loop equal the oracle's DA, element by element
    E = _read(pre + ".elem")
    oda = oracle.DA(bal, 30)
    assert np.array_equal(E[:, :3], bal[:, :3])
    assert np.array_equal(E[:, 3] & 255, bal[:, 3] + 1)
    assert np.array_equal(E[:, 4:].reshape(-1, 8, 3), oda.node_xyz[oda.nodes])
    # MatShell callbacks give what the direct calls give (the element loop
    # adds shared node runs atomically, so repeated FP64 calls agree to
    # rounding, not bit for bit)
    tol = 1e-13 * info["ymax"]
    assert info["shell_err"] <= tol and info["diag_err"] <= tol
    assert abs(info["mass_sum"] - 1.0) < 1e-12
    assert info["dir_err"] <= tol and info["dirdiag_err"] <= tol and info["mg_levels"] >= 2
    # SFC_treeSort(TS_REMOVE_DUPLICATES) of the messy copy gives back the balanced octree
    assert np.array_equal(_read(pre + ".sorted"), bal) and info["inplace_sorted"] == 1
