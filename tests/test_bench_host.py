"""bench.py's host-side helpers without a GPU: the roofline peak it reads,
the clock-sample summary, the per-kernel tables and the reference arm's
sample."""
import json

import bench


def test_peak_is_the_measured_copy_rate(tmp_path, monkeypatch):
    peak, kind = bench._peaks()
    try:
        with open(bench.os.path.join(bench.ROOT, "MEASURED_PEAKS.json")) as f:
            want = float(json.load(f)["hbm_gbs"])
        assert (peak, kind) == (want, "measured")
    except FileNotFoundError:
        assert (peak, kind) == (6800.0, "fallback")
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))  # no file: the stated fallback
    assert bench._peaks() == (6800.0, "fallback")


class _DoneProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_summary():
    cs = bench.ClockSampler(0)
    cs.proc = _DoneProc()
    cs.rows = [["2070", "2070", "900", "0x0", "Not Active", "Not Active", "Not Active", "Not Active", "100"],
               ["2040", "2070", "1380", "0x4", "Not Active", "Not Active", "Not Active", "Active", "96"],
               ["2055", "2070", "1200", "0x0", "Not Active", "Not Active", "Not Active", "Not Active", "98"],
               ["garbage"]]
    s = cs.stop()
    assert s == {"sm_mhz": 2055.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3,
                 "gpu_util_pct_mean": 98.0}
    # a sample without the utilisation column still counts for the clocks
    cs.rows = [["2070", "2070", "900", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"]]
    s = cs.stop()
    assert (s["samples"], s["gpu_util_pct_mean"]) == (1, None)


def test_kernel_tables():
    a = {"k1": (10.0, 2, 100.0), "k2": (1.0, 1, 5.0)}
    b = {"k1": (5.0, 1, 50.0), "k3": (7.0, 3, 0.0)}
    m = bench._merge_stats([a, b])
    assert m == {"k1": (15.0, 3, 150.0), "k2": (1.0, 1, 5.0), "k3": (7.0, 3, 0.0)}
    top = bench._top_kernels({k: (v[0], v[1]) for k, v in m.items()}, k=2)
    assert list(top) == ["k1", "k3"] and top["k1"] == [15.0, 3]
    # with algorithmic bytes: GB/s = bytes / (ms * 1e6); none without bytes
    top = bench._top_kernels({"k1": (2.0, 4, 3e9), "k3": (1.0, 1, 0.0)})
    assert top == {"k1": [2.0, 4, 1500.0], "k3": [1.0, 1, None]}


def test_reference_sample_fills_the_cores():
    tasks = bench._ref_tasks(16)
    small = [r for r in bench._stream() if len(r.points) <= bench.REF_MAX_POINTS]
    assert len(small) >= 1 and len(tasks) == max(16, len(small))
    assert all(len(r.points) <= bench.REF_MAX_POINTS for r in tasks)
    assert [r.rid for r in tasks[: len(small)]] == [r.rid for r in small]
    before = bench.os.environ.get("OPENBLAS_NUM_THREADS")
    with bench._one_thread_per_process():
        assert bench.os.environ["OPENBLAS_NUM_THREADS"] == "1"
    assert bench.os.environ.get("OPENBLAS_NUM_THREADS") == before  # restored
