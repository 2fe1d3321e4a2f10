"""The reference-written point and octree files (tests/golden/io, made by
tests/golden/make_golden.py from the reference's own writePtsToFile,
writeNodesToFile and writeNodesToFile_binary) agree with the oracle's octree
for the same points, and the library's header-only point count reads them
(no GPU needed)."""
import ctypes
import json
import os

import numpy as np

from dendro_gb300 import _lib

HERE = os.path.join(os.path.dirname(__file__), "golden", "io")


def _parse_text(path):
    tok = open(path).read().split()
    dim, depth, n = int(tok[0]), int(tok[1]), int(tok[2])
    return dim, depth, np.array(tok[3:3 + 4 * n], np.uint64).astype(np.uint32).reshape(n, 4)


def test_fixtures_match_the_oracle(oracle):
    pts = np.load(os.path.join(HERE, "gauss200_points.npy"))
    raw = open(os.path.join(HERE, "gauss200.pts"), "rb").read()
    assert int(np.frombuffer(raw[:4], np.uint32)[0]) == len(pts)
    assert np.array_equal(np.frombuffer(raw[4:], np.float64).reshape(-1, 3), pts)
    want = oracle.balance(oracle.points_to_octree(pts, 30, 1), 30)
    dim, depth, text = _parse_text(os.path.join(HERE, "gauss200.ot"))
    assert (dim, depth) == (3, 30)
    assert np.array_equal(text, want)
    rec = np.fromfile(os.path.join(HERE, "gauss200.otb"), np.uint32).reshape(-1, 7)
    assert np.array_equal(rec[:, :4], want)
    assert (rec[:, 4] == 1).all() and (rec[:, 5] == 3).all() and (rec[:, 6] == 30).all()
    info = json.load(open(os.path.join(HERE, "gauss200.json")))
    # the reference's binary reader returns one record more than the file holds
    assert info["binary_read"] == len(want) + 1 and info["text_read"] == len(want)


def test_point_count_from_the_header():
    L = _lib.load()
    n = ctypes.c_size_t()
    assert L.dg_pts_file_count(os.path.join(HERE, "gauss200.pts").encode(), ctypes.byref(n)) == 0
    assert n.value == 200
    assert L.dg_pts_file_count(b"/nonexistent/file.pts", ctypes.byref(n)) == 1
