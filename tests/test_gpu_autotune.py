"""The radix sort's autotuner: the first sort of a size class times the
onesweep launch shapes (keys per thread x blocks per SM) and the
digit-histogram grid, keeps the fastest, and stores the decision in the
disk cache; a new process on the same device reads it back instead of
tuning again.  Results are the same whichever shape runs."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, {root!r})
import numpy as np
import dendro_gb300 as dg
from dendro_gb300 import datagen
ctx = dg.Context(0)
pts = datagen.lognormal(300_000, seed=5)
out = dg.sortUniquePoints(pts, ctx=ctx)
np.save({out!r}, out)
print(ctx.autotune_log())
"""


def _run(tmp_path, cache, tag):
    out = tmp_path / f"{tag}.npy"
    env = dict(os.environ, DENDRO_GB300_TUNE_CACHE=str(cache))
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT, out=str(out))], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout, np.load(out)


def test_decisions_are_tuned_then_read_from_the_disk_cache(tmp_path):
    cache = tmp_path / "tune" / "autotune.tsv"
    log1, a = _run(tmp_path, cache, "first")
    assert "keys/thread x blocks/SM" in log1 and "histogram blocks/SM" in log1
    lines = cache.read_text().splitlines()
    assert lines and all(len(ln.split("\t")) == 6 for ln in lines)
    dev = lines[0].split("\t")[0]
    assert "GB300" in dev or "|cc" in dev
    log2, b = _run(tmp_path, cache, "second")
    assert "(disk cache)" in log2 and "keys/thread x blocks/SM" not in log2
    assert np.array_equal(a, b)
    # a corrupt cache line is ignored, not trusted
    cache.write_text("garbage\n" + "\t".join([dev, "1", "18", "999", "9", "3"]) + "\n")
    log3, c = _run(tmp_path, cache, "third")
    assert np.array_equal(a, c) and "keys/thread x blocks/SM" in log3
