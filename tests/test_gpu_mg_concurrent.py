"""Multigrid solves running at the same time on several contexts (threads,
streams) give the results they give one at a time: the same iteration
counts (within one) and the 1e-8 residual.  Catches races inside the element
loop that a single context rarely shows (a block reading shared memory
before it is filled, state shared across contexts)."""
import threading

import numpy as np
import pytest

import dendro_gb300 as dg
from dendro_gb300 import datagen, serving

pytestmark = pytest.mark.gpu


def _solve_all(ctx, reqs, out):
    import torch

    for r in reqs:
        lin = dg.points2Octree(r.points, ctx=ctx)
        bal = dg.balanceOctree(lin)
        lin.free()
        mg = dg.MultiGrid(bal, max_coarse_elems=4096, ctx=ctx)
        bal.free()
        f = datagen.bumps(mg.level_nodes(0, device=True))
        b = mg.rhs(f)
        x, it, rr = mg.solve(b, precision=32, rtol=1e-8, maxit=50)
        out[r.rid] = (it, rr, float(torch.linalg.vector_norm(x)))
        mg.free()


def test_concurrent_solves_equal_sequential():
    pytest.importorskip("torch")
    reqs = serving.poisson_stream(9, rate=400.0, lo=2e3, hi=2e5, seed=7)
    ctx = dg.Context(0)
    ref = {}
    _solve_all(ctx, reqs, ref)
    ctx.close()
    for k, (it, rr, _) in ref.items():
        assert rr <= 1e-8, (k, it, rr)
    for _ in range(2):
        ctxs = [dg.Context(0) for _ in range(3)]
        outs = [{} for _ in ctxs]
        threads = [threading.Thread(target=_solve_all, args=(c, reqs[i::3] + reqs, o))
                   for i, (c, o) in enumerate(zip(ctxs, outs))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for c in ctxs:
            c.close()
        for o in outs:
            assert set(o) == set(ref)
            for k, (it, rr, xn) in o.items():
                assert rr <= 1e-8 and abs(it - ref[k][0]) <= 1, (k, it, rr, ref[k])
                assert abs(xn - ref[k][2]) <= 1e-6 * ref[k][2]
