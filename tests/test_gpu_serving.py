"""Serving: every request's result is the same served in a continuous batch
as through the plain per-call path, and the admission budget is respected.

"The same" is checked on the results themselves: each request's balanced
octree records are bit-identical, and its FP64 solution, matched node by
node through the node coordinates, agrees with the plain path's within
SOLUTION_RTOL (both solves stop at an FP64 relative residual of 1e-8; the
FP32 V-cycle adds shared node runs atomically, so two solves agree to the
solver tolerance, not bit for bit).  One request is also solved by the
oracle's FP64 multigrid (oracle/mg_ref.py) and compared the same way."""
import numpy as np
import pytest

from dendro_gb300 import datagen, serving

pytestmark = pytest.mark.gpu

SOLUTION_RTOL = 1e-6


def _stream():
    return serving.poisson_stream(14, rate=400.0, lo=2e3, hi=3e5, seed=7)


def _by_coords(xyz, v):
    """The values ordered by node coordinates (x, then y, then z)."""
    order = np.lexsort(np.asarray(xyz).T[::-1])
    return np.asarray(xyz)[order], np.asarray(v)[order]


def _same_solution(ra, rb, rtol):
    xa, va = _by_coords(ra.node_xyz, ra.solution)
    xb, vb = _by_coords(rb.node_xyz, rb.solution)
    assert np.array_equal(xa, xb), f"request {ra.rid}: node sets differ"
    err = np.linalg.norm(va - vb) / np.linalg.norm(va)
    assert err <= rtol, f"request {ra.rid}: solutions differ by {err:.2e}"
    return err


@pytest.fixture(scope="module")
def served_and_plain():
    plain = serving.PlainServer(solve_maxit=50, keep="octree,solution")
    a = plain.run(_stream())
    plain.close()
    srv = serving.BatchingServer(workers=3, solve_maxit=50, keep="octree,solution")
    b = srv.run(_stream())
    srv.close()
    assert max(srv.batches) > 1  # requests really were batched
    return sorted(a, key=lambda r: r.rid), sorted(b, key=lambda r: r.rid)


def test_served_equals_plain(served_and_plain):
    a, b = served_and_plain
    errs = []
    for ra, rb in zip(a, b):
        assert not ra.error and not rb.error, (ra.error, rb.error)
        assert np.array_equal(ra.octree, rb.octree), f"request {ra.rid}: balanced octrees differ"
        assert (ra.n_octants, ra.n_balanced) == (rb.n_octants, rb.n_balanced) and len(ra.octree) == ra.n_balanced
        assert ra.relres <= 1e-8 and rb.relres <= 1e-8
        errs.append(_same_solution(ra, rb, SOLUTION_RTOL))
        assert rb.t_done >= rb.t_built >= rb.t_admit >= rb.arrival - 1e-3
    print("served vs plain solution differences: max %.2e" % max(errs))


def test_comparison_catches_wrong_results(served_and_plain):
    """The comparison itself fails on a corrupted octree or a permuted
    solution (checked on a copy of the results)."""
    a, b = served_and_plain
    ra, rb = a[3], b[3]
    bad = rb.octree.copy()
    bad[len(bad) // 2, 3] += 1
    assert not np.array_equal(ra.octree, bad)
    perm = serving.Request(rb.rid, rb.arrival, rb.points, node_xyz=rb.node_xyz,
                           solution=np.roll(rb.solution, 1))
    with pytest.raises(AssertionError):
        _same_solution(ra, perm, SOLUTION_RTOL)


def test_one_request_against_the_oracle_solve(served_and_plain, oracle):
    from oracle.mg_ref import OracleMG

    _, b = served_and_plain
    r = min(b, key=lambda q: len(q.points))
    assert np.array_equal(r.octree, oracle.balance(oracle.points_to_octree(r.points, 30, 1), 30))
    mg = OracleMG(r.octree, 30, max_coarse=4096)
    f = datagen.bumps(mg.das[0].node_xyz)
    x, it, rr = mg.solve(mg.rhs(f), rtol=1e-8, maxit=50)
    assert rr <= 1e-8
    ref = serving.Request(r.rid, 0.0, r.points, node_xyz=mg.das[0].node_xyz, solution=x)
    _same_solution(ref, r, SOLUTION_RTOL)


def test_admission_budget_serialises_large_requests():
    reqs = _stream()[:6]
    # a budget below every request's estimate: each is admitted alone, once the device is empty
    need = min(serving.estimate_bytes(len(r.points)) for r in reqs) - 1
    srv = serving.BatchingServer(workers=2, hbm_budget=need, solve_maxit=20)
    out = srv.run(reqs)
    srv.close()
    # with room for one request at a time nothing was batched or overlapped
    assert max(srv.batches) == 1
    done = sorted(out, key=lambda r: r.t_admit)
    for prev, nxt in zip(done, done[1:]):
        assert nxt.t_admit >= prev.t_done - 1e-3
    s = serving.summarize(out, max(r.t_done for r in out))
    assert s["errors"] == 0 and s["p99_ms"] >= s["p50_ms"] > 0
