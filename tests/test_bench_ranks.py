"""The multi-process path of bench.py (replicas only: one process per GPU,
no data-path collective): two gloo ranks on the CPU check the slowest-rank
reduction and the whole-job value the bench reports, and the rank
environment it reads.  CPU only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, got_local = bench._dist()
        ms, e2e = 100.0 + 10 * rank, 150.0 - 20 * rank  # rank 1 slower on one, faster on the other
        m, e = bench.max_over_ranks([ms, e2e], "cpu")
        q.put((rank, got_ws, got_rank, got_local, m, e, bench.replica_value(ws, 1_000_000, m)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ws, r, local, m, e, v in out:
        assert (ws, r, local) == (2, rank, rank)
        assert (m, e) == (110.0, 150.0)  # element-wise maximum over the ranks
        assert v == pytest.approx(2 * 1_000_000 / 0.110 / 1e6)


def test_single_rank_is_unchanged():
    import bench

    assert bench.max_over_ranks([1.5, 2.5], "cpu") == [1.5, 2.5]
    assert bench.replica_value(1, 2_000_000, 500.0) == pytest.approx(4.0)
