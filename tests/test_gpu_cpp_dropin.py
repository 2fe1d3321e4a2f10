"""The C++ drop-in mirror (include/dendro_gb300.hpp) compiled by a C++ caller,
run on the GPU and checked against the oracle."""
import json
import os
import subprocess

import numpy as np
import pytest

from dendro_gb300 import build as cuda_build
from dendro_gb300 import datagen

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_dropin(oracle, tmp_path):
    lib = cuda_build.build()
    exe = tmp_path / "dropin"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp"), "-o", str(exe),
                           lib, "-Wl,-rpath," + os.path.dirname(lib)])
    pts = datagen.gaussian(20000, 0.5, 0.1, seed=41)
    pf, of = tmp_path / "p.pts", tmp_path / "b.oct"
    with open(pf, "wb") as f:
        f.write(np.uint64(len(pts)).tobytes())
        f.write(pts.tobytes())
    r = subprocess.run([str(exe), str(pf), str(of)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    info = json.loads(r.stdout.strip().splitlines()[-1])
    b = open(of, "rb").read()
    bal = np.frombuffer(b[8:], np.uint32).reshape(-1, 4)
    ref = oracle.balance(oracle.points_to_octree(pts, 30, 1), 30)
    assert np.array_equal(bal, ref)
    assert info["n_elem"] == len(ref)
    assert info["n_node"] == oracle.DA(ref, 30).n_node
    # mass matrix applied to ones sums to the domain volume
    assert abs(info["sum_A1"] - 1.0) < 1e-12
    assert info["n_coarse"] == len(oracle.coarsen(ref, 30))
    sub = ref[::-1][::5]
    assert info["n_complete_sub"] == len(oracle.complete(sub, 30, 0, 0))
    assert info["complete_bal_same"] == 1
    assert info["sort_ok"] == 1
    # A 1 from the CSR rows, the diagonal and the per-element form agree with
    # the matVec, relative to the largest entry (FP64 rounding only)
    assert info["mat_err"] < 1e-12 and info["diag_err"] < 1e-12 and info["coef_err"] < 1e-12
