"""Serving: every request's result is the same served in a continuous batch
as through the plain per-call path (octrees exactly; the FP32-V-cycle solve
to the same FP64 residual bound), and the admission budget is respected."""
import numpy as np
import pytest

from dendro_gb300 import serving

pytestmark = pytest.mark.gpu


def _stream():
    return serving.poisson_stream(14, rate=400.0, lo=2e3, hi=3e5, seed=7)


def test_served_equals_plain():
    plain = serving.PlainServer(solve_maxit=50)
    a = plain.run(_stream())
    plain.close()
    srv = serving.BatchingServer(workers=3, solve_maxit=50)
    b = srv.run(_stream())
    srv.close()
    assert max(srv.batches) > 1  # requests really were batched
    for ra, rb in zip(sorted(a, key=lambda r: r.rid), sorted(b, key=lambda r: r.rid)):
        assert not ra.error and not rb.error, (ra.error, rb.error)
        assert (ra.n_octants, ra.n_balanced) == (rb.n_octants, rb.n_balanced)
        assert ra.relres <= 1e-8 and rb.relres <= 1e-8
        assert abs(ra.iterations - rb.iterations) <= 1
        assert abs(ra.solution_norm - rb.solution_norm) <= 1e-6 * ra.solution_norm
        assert rb.t_done >= rb.t_built >= rb.t_admit >= rb.arrival - 1e-3


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
