"""Point and octree files through the GPU path: bytes written equal the
reference's own files, files read give the reference's octants, and round
trips hold at sizes that cross the 32 MB staging buffers."""
import os

import numpy as np
import pytest

import dendro_gb300 as dg
from dendro_gb300 import DendroError, datagen

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(__file__), "golden", "io")


def _bytes(path):
    with open(path, "rb") as f:
        return f.read()


def test_writers_reproduce_the_reference_files(ctx, tmp_path):
    pts = np.load(os.path.join(HERE, "gauss200_points.npy"))
    dg.writePtsToFile(tmp_path / "a.pts", pts, ctx=ctx)
    assert _bytes(tmp_path / "a.pts") == _bytes(os.path.join(HERE, "gauss200.pts"))
    bal = dg.balanceOctree(dg.points2Octree(pts, ctx=ctx))
    dg.writeNodesToFile(tmp_path / "a.ot", bal)
    assert _bytes(tmp_path / "a.ot") == _bytes(os.path.join(HERE, "gauss200.ot"))
    dg.writeNodesToFile_binary(tmp_path / "a.otb", bal)
    assert _bytes(tmp_path / "a.otb") == _bytes(os.path.join(HERE, "gauss200.otb"))


def test_readers_give_the_reference_octants(ctx):
    want = np.fromfile(os.path.join(HERE, "gauss200.otb"), np.uint32).reshape(-1, 7)[:, :4]
    t = dg.readNodesFromFile(os.path.join(HERE, "gauss200.ot"), ctx=ctx)
    assert np.array_equal(t.to_numpy(), want) and t.max_depth == 30
    b = dg.readNodesFromFile_binary(os.path.join(HERE, "gauss200.otb"), ctx=ctx)
    assert np.array_equal(b.to_numpy(), want)  # the file's records, no repeated last one
    pts = np.load(os.path.join(HERE, "gauss200_points.npy"))
    assert np.array_equal(dg.readPtsFromFile(os.path.join(HERE, "gauss200.pts"), ctx=ctx), pts)
    dev = dg.readPtsFromFile(os.path.join(HERE, "gauss200.pts"), device=True, ctx=ctx)
    assert np.array_equal(dev.cpu().numpy(), pts)


def test_round_trips_across_staging_chunks(ctx, tmp_path):
    torch = pytest.importorskip("torch")
    pts = datagen.lognormal(3_000_000, seed=21)  # 72 MB: three staging chunks
    dev = torch.from_numpy(pts).cuda()
    dg.writePtsToFile(tmp_path / "big.pts", dev, ctx=ctx)
    back = dg.readPtsFromFile(tmp_path / "big.pts", device=True, ctx=ctx)
    assert torch.equal(back, dev)
    assert np.array_equal(dg.readPtsFromFile(tmp_path / "big.pts", ctx=ctx), pts)
    bal = dg.balanceOctree(dg.points2Octree(dev[:400_000].contiguous(), ctx=ctx))
    want = bal.to_numpy()
    dg.writeNodesToFile(tmp_path / "big.ot", bal)
    assert os.path.getsize(tmp_path / "big.ot") > (40 << 20)
    assert np.array_equal(dg.readNodesFromFile(tmp_path / "big.ot", ctx=ctx).to_numpy(), want)
    dg.writeNodesToFile_binary(tmp_path / "big.otb", bal)
    assert np.array_equal(dg.readNodesFromFile_binary(tmp_path / "big.otb", ctx=ctx).to_numpy(), want)
    # the text lines equal a host formatting of the same octants
    head = open(tmp_path / "big.ot").read(4096).splitlines()
    assert head[0] == "3 30" and head[1] == str(len(want))
    assert head[2] == " ".join(str(v) for v in want[0])


def test_malformed_files_are_refused(ctx, tmp_path):
    (tmp_path / "bad.ot").write_text("3 30\n2\n0 0 0 1\n536870912 0 0 x\n")
    with pytest.raises(DendroError):
        dg.readNodesFromFile(tmp_path / "bad.ot", ctx=ctx)
    (tmp_path / "short.ot").write_text("3 30\n2\n0 0 0 1\n")
    with pytest.raises(DendroError):
        dg.readNodesFromFile(tmp_path / "short.ot", ctx=ctx)
    (tmp_path / "big.ot").write_text("3 30\n1\n0 0 0 99999999999\n")
    with pytest.raises(DendroError):
        dg.readNodesFromFile(tmp_path / "big.ot", ctx=ctx)
    (tmp_path / "odd.otb").write_bytes(b"\0" * 30)
    with pytest.raises(DendroError):
        dg.readNodesFromFile_binary(tmp_path / "odd.otb", ctx=ctx)
    raw = _bytes(os.path.join(HERE, "gauss200.pts"))
    (tmp_path / "cut.pts").write_bytes(raw[:1000])
    with pytest.raises(DendroError):
        dg.readPtsFromFile(tmp_path / "cut.pts", ctx=ctx)
    dg.writePtsToFile(tmp_path / "none.pts", np.zeros((0, 3)), ctx=ctx)
    assert os.path.getsize(tmp_path / "none.pts") == 0  # as the reference: nothing written
    assert len(dg.readPtsFromFile(tmp_path / "none.pts", ctx=ctx)) == 0
