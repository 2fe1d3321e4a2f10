"""Host logic of the serving module without a GPU: admission by the HBM
budget (arrival order, the lone oversized request, the batch point cap),
the byte estimate, the seeded request stream and the latency summary."""
import numpy as np

from dendro_gb300 import serving


def _req(i, n):
    return serving.Request(i, 0.01 * i, np.zeros((n, 3)))


def test_estimate_grows_with_points():
    a, b = serving.estimate_bytes(1000), serving.estimate_bytes(2000)
    assert 0 < a < b and b - a == serving.estimate_bytes(3000) - b


def test_admit_in_arrival_order_within_budget():
    sizes = [100_000, 200_000, 300_000, 50_000]
    budget = serving.estimate_bytes(100_000) + serving.estimate_bytes(200_000)
    waiting = [_req(i, n) for i, n in enumerate(sizes)]
    batch, inflight = serving.admit(waiting, 0, budget, 10**9)
    assert [r.rid for r, _ in batch] == [0, 1]          # the third would pass the budget
    assert inflight == sum(b for _, b in batch) <= budget
    assert [r.rid for r in waiting] == [2, 3]            # no overtaking: 3 waits behind 2
    batch, inflight2 = serving.admit(waiting, inflight, budget, 10**9)
    assert batch == [] and inflight2 == inflight


def test_lone_oversized_request_is_admitted_when_idle():
    waiting = [_req(0, 5_000_000), _req(1, 10)]
    batch, inflight = serving.admit(waiting, 0, 1, 10**9)
    assert [r.rid for r, _ in batch] == [0] and inflight == serving.estimate_bytes(5_000_000)
    batch, _ = serving.admit(waiting, inflight, 1, 10**9)
    assert batch == []                                   # not while something is in flight


def test_batch_point_cap():
    waiting = [_req(i, 400) for i in range(5)]
    batch, _ = serving.admit(waiting, 0, 10**15, 1000)
    assert [r.rid for r, _ in batch] == [0, 1]


def test_stream_is_seeded_and_summary_reads_latencies():
    a = serving.poisson_stream(6, rate=100.0, lo=1e4, hi=2e4, seed=7)
    b = serving.poisson_stream(6, rate=100.0, lo=1e4, hi=2e4, seed=7)
    assert [len(r.points) for r in a] == [len(r.points) for r in b]
    assert all(np.array_equal(x.points, y.points) for x, y in zip(a, b))
    assert all(a[i].arrival < a[i + 1].arrival for i in range(5))
    for i, r in enumerate(a):
        r.t_done = r.arrival + 0.1 * (i + 1)
    s = serving.summarize(a, wall=1.0)
    assert s["requests"] == 6 and s["errors"] == 0
    assert abs(s["p50_ms"] - 350.0) < 1e-6
    assert s["Mpts_per_s"] == sum(len(r.points) for r in a) / 1e6
