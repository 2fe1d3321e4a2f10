"""Benchmark of the octree hot path on one GB300, on the metric
"served vs plain Mpts/s + p99 ms; FP32-MG vs FP64 solve time @1e-8 rel res".

Headline workload (serving): a stream of SERVE_REQUESTS requests with
Poisson arrivals (mean 200 req/s, seed 4), cloud sizes log-uniform in
[1e4, 8e6], alternately Gaussian-mixture and log-normal clouds, FP64
coordinates.  Each request is points2Octree -> balanceOctree(incCorner) ->
mesh (ot::DA) -> multigrid set-up -> CG with an FP32 V-cycle (FP64
residuals) to 1e-8 relative residual, at most 50 iterations.  One step = the
whole stream served once by the continuous-batching server
(dendro_gb300.serving.BatchingServer).

  value : served Mpts/s with every cloud already resident in HBM
  e2e   : the same stream served from host (pinned) clouds through the C ABI,
          each request's points copied in and its result read back inside
          the timed region
  plain : the same stream through the per-call drop-in (PlainServer: one
          request at a time, one call per reference function)
  p50 / p99 request latency (arrival -> result) for both servers.

Also reported, each as its own block:
  precision : the Poisson workload (16e6 N(0.5, 0.15^2) points, seed 3):
              FP32-V-cycle vs all-FP64 solve time to 1e-8, per-kernel times
  batching  : 256 Gaussian-mixture clouds (sizes log-uniform in [1e4, 4e6],
              seed 2) built and balanced in one segmented pass vs one call
              per cloud
  scale     : 64e6 log-normal points (seed 0): build+balance Mpts/s with
              the per-kernel roofline, the mesh build and the Laplacian+mass
              matVec (FP32 / FP64) on the balanced octree
nvidia-smi clocks are sampled during the timed region.

--impl reference serves a bounded sample of the same stream on the host
cores with the CPU restatement of the reference path (oracle/: C for the
octree and mesh, numpy for the FP64 multigrid solve), one request per
process.

Multi-GPU: replicas only (the path has no exchange step): each rank serves
its own copy of the stream; value sums the ranks' points over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "served vs plain Mpts/s + p99 ms; FP32-MG vs FP64 solve time @1e-8 rel res"
SERVE_REQUESTS = 32
SERVE_RATE = 200.0
SERVE_SIZES = (1e4, 8e6)
SERVE_SEED = 4
SOLVE_MAXIT = 50
REF_MAX_POINTS = 40_000  # reference arm: requests of the stream up to this size


def _traffic_ratios() -> dict:
    """DRAM bytes per algorithmic byte of a kernel, from one ncu capture each
    (profiles/dram_traffic.txt: name, DRAM bytes, algorithmic bytes).  The
    traffic grows with the elements / keys a launch processes, so the ratio
    scales it to the bench's average launch."""
    out = {}
    try:
        for line in open(os.path.join(ROOT, "profiles", "dram_traffic.txt")):
            f = line.split()
            if f and not line.startswith("#") and len(f) >= 3:
                out[f[0]] = float(f[1]) / float(f[2])
    except OSError:
        pass
    return out


TRAFFIC_PER_ALG_BYTE = _traffic_ratios()


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons in the background."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return

        def reader():
            for line in self.proc.stdout:
                self.rows.append([c.strip() for c in line.split(",")])

        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, util, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax.append(float(r[1]))
                for nm, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(nm)
                util.append(float(r[8]))
            except (ValueError, IndexError):
                continue
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
            # nvidia-smi's utilization.gpu: the share of each sample period in
            # which some kernel ran (not how many SMs it kept busy)
            "gpu_util_pct_mean": statistics.mean(util) if util else None,
        }


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(vals, device) -> list:
    """The element-wise maximum of vals over all ranks (the slowest
    replica's times); vals unchanged at one rank."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return [float(v) for v in vals]
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def replica_value(ws: int, points_per_replica: int, ms: float) -> float:
    """Whole-job Mpts/s of ws replicas that each served points_per_replica
    points, over the slowest replica's time."""
    return ws * points_per_replica / (ms * 1e-3) / 1e6


def _top_kernels(stats: dict, k: int = 10) -> dict:
    """{kernel: [total ms, launches]} of the k kernels with the most time;
    where the statistics carry each kernel's algorithmic bytes, a third
    entry gives its achieved GB/s (bytes over event time)."""
    top = sorted(stats.items(), key=lambda kv: -kv[1][0])[:k]
    out = {}
    for name, v in top:
        row = [round(v[0], 3), int(v[1])]
        if len(v) > 2:
            row.append(round(v[2] / (v[0] * 1e6), 1) if v[0] > 0 and v[2] > 0 else None)
        out[name] = row
    return out


def _merge_stats(parts) -> dict:
    out = {}
    for st in parts:
        for k, (ms, cnt, b) in st.items():
            o = out.get(k, (0.0, 0, 0.0))
            out[k] = (o[0] + ms, o[1] + cnt, o[2] + b)
    return out


def _stream(count: int = SERVE_REQUESTS):
    from dendro_gb300 import serving

    return serving.poisson_stream(count, rate=SERVE_RATE, lo=SERVE_SIZES[0], hi=SERVE_SIZES[1],
                                  seed=SERVE_SEED)


# ---------------------------------------------------------------------------
# reference arm (CPU)
# ---------------------------------------------------------------------------
def cpu_request_run(args):
    """One request of the stream on the CPU restatement (worker process):
    points2Octree + balanceOctree + DA (oracle C), then the FP64 multigrid
    CG (oracle numpy) on the same right-hand side as the GPU path."""
    rid, pts, maxit = args
    sys.path.insert(0, ROOT)
    from dendro_gb300 import datagen
    from oracle import dg_oracle
    from oracle.mg_ref import OracleMG

    t0 = time.perf_counter()
    lin = dg_oracle.points_to_octree(pts, 30, 1)
    bal = dg_oracle.balance(lin, 30)
    mg = OracleMG(bal, 30, max_coarse=4096)
    f = datagen.bumps(mg.das[0].node_xyz)
    b = mg.rhs(f)
    _, it, rr = mg.solve(b, rtol=1e-8, maxit=maxit)
    return rid, time.perf_counter() - t0, len(pts), it, rr


class _one_thread_per_process:
    """Worker processes started inside this block run one thread each
    (numpy's BLAS would otherwise start a thread pool per process and
    oversubscribe the cores); the caller's environment is restored after."""

    VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")

    def __enter__(self):
        self.saved = {v: os.environ.get(v) for v in self.VARS}
        for v in self.VARS:
            os.environ[v] = "1"

    def __exit__(self, *exc):
        for v, old in self.saved.items():
            if old is None:
                os.environ.pop(v, None)
            else:
                os.environ[v] = old


def _ref_tasks(cores: int):
    """The reference arm's sample: the stream's requests of at most
    REF_MAX_POINTS points, repeated in turn so that every host core serves
    one of them per step (a request per process, as one MPI rank each)."""
    small = [r for r in _stream() if len(r.points) <= REF_MAX_POINTS]
    n = max(cores, len(small)) if small else 0
    return [small[i % len(small)] for i in range(n)]


def run_reference(args):
    """CPU arm: the requests of the stream with at most REF_MAX_POINTS points,
    each served by the oracle on its own host core, all at once per step."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import multiprocessing as mp

    from oracle import dg_oracle

    dg_oracle.build()
    reqs = _ref_tasks(os.cpu_count() or 1)
    cores = min(os.cpu_count() or 1, max(len(reqs), 1))
    npts = sum(len(r.points) for r in reqs)
    ctxmp = mp.get_context("spawn")
    times, lat = [], []
    with _one_thread_per_process():
        pool = ctxmp.Pool(cores)
    with pool:
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(cpu_request_run, [(r.rid, r.points, SOLVE_MAXIT) for r in reqs])
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                times.append(dt)
                lat.extend(1e3 * r[1] for r in res)
    ms = 1e3 * sum(times) / len(times)
    value = npts / (ms * 1e-3) / 1e6
    lat.sort()
    sample = (f"{len(reqs)} requests ({npts} points): the serving stream's requests with <= {REF_MAX_POINTS} "
              f"points, repeated to fill {cores} host cores, one per process: oracle C points2Octree + "
              f"balanceOctree + DA per level, numpy FP64 multigrid CG to 1e-8 (<= {SOLVE_MAXIT} iterations)")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "Mpts/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int keys, FP64 coords and solve",
        "data": "synthetic",
        "config": {"workload": "serving stream (bounded CPU sample)", "requests": len(reqs), "points": npts,
                   "max_depth": 30, "max_pts_per_octant": 1, "rate_req_s": SERVE_RATE, "seed": SERVE_SEED},
        "p50_ms": lat[len(lat) // 2] if lat else None,
        "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))] if lat else None,
        "cpu_baseline": {"value": value, "unit": "Mpts/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(cores: int) -> dict:
    """The reference arm's measurement, short (1 warm-up + 1 timed pass), for
    the cpu_baseline key of the GPU line."""
    import multiprocessing as mp

    from oracle import dg_oracle

    dg_oracle.build()
    reqs = _ref_tasks(cores)
    cores = min(cores, max(len(reqs), 1))
    npts = sum(len(r.points) for r in reqs)
    with _one_thread_per_process():
        pool = mp.get_context("spawn").Pool(cores)
    with pool:
        pool.map(cpu_request_run, [(r.rid, r.points, SOLVE_MAXIT) for r in reqs])
        t0 = time.perf_counter()
        pool.map(cpu_request_run, [(r.rid, r.points, SOLVE_MAXIT) for r in reqs])
        dt = time.perf_counter() - t0
    return {"value": npts / dt / 1e6, "unit": "Mpts/s", "cores": cores, "kind": "port",
            "sample": f"{len(reqs)} requests ({npts} points): the serving stream's requests with <= {REF_MAX_POINTS} "
                      f"points, repeated to fill {cores} host cores, one per process: oracle C octree + DA, numpy "
                      f"FP64 multigrid CG to 1e-8; {dt:.2f} s"}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def _latency(out) -> dict:
    lat = sorted(1e3 * r.latency for r in out)
    return {"p50_ms": lat[len(lat) // 2], "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))]}


def run_serving(args, local, barrier):
    """The headline: the stream served by BatchingServer (device-resident and
    host clouds) and by PlainServer."""
    import numpy as np
    import torch

    from dendro_gb300 import serving

    host = _stream(args.serve_requests)
    npts = sum(len(r.points) for r in host)
    dev = f"cuda:{local}"
    on_dev = [torch.from_numpy(r.points).to(dev) for r in host]
    pinned = [torch.from_numpy(r.points).pin_memory() for r in host]
    torch.cuda.synchronize()

    def replay(srv, clouds):
        reqs = [serving.Request(r.rid, r.arrival, c) for r, c in zip(host, clouds)]
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = srv.run(reqs)
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    srv = serving.BatchingServer(device=local, workers=args.serve_workers, solve_maxit=SOLVE_MAXIT)
    for _ in range(args.warmup):
        replay(srv, on_dev)
    ctxs = [srv.ctx] + srv.worker_ctx
    sampler = ClockSampler(local)
    sampler.start()
    walls, outs = [], []
    srv.build_s.clear()
    for _ in range(args.steps):
        out, wall = replay(srv, on_dev)
        walls.append(wall)
        outs.extend(out)
    served_build_s = sum(srv.build_s) / args.steps
    clocks = sampler.stop()
    # per-kernel device times: one more replay of the same stream with every
    # launch bracketed by CUDA events on its stream (the timed steps above run
    # without them, with the CG iterations replayed from CUDA graphs)
    for c in ctxs:
        c.profile(True)
    replay(srv, on_dev)
    stats = _merge_stats(c.profile_stats() for c in ctxs)
    for c in ctxs:
        c.profile(False)
    batches = list(srv.batches)
    # the same stream from pinned host memory: every request's points copied
    # in, and its FP64 solution vector copied back to pinned host memory
    e2e_walls, d2h = [], 0
    if not args.skip_e2e:
        srv.keep = "solution"
        replay(srv, pinned)
        for _ in range(args.steps):
            out_e, wall = replay(srv, pinned)
            e2e_walls.append(wall)
        d2h = sum(r.solution.nbytes for r in out_e)
        assert all(r.solution is not None and len(r.solution) > 0 for r in out_e)
        srv.keep = ""
    # the reference arm's own sample (the stream's requests of at most
    # REF_MAX_POINTS points, as many as the host has cores), all arriving at
    # once, so the CPU and GPU figures compare the same inputs
    same = _ref_tasks(os.cpu_count() or 1)
    same_pts = sum(len(r.points) for r in same)
    same_dev = [torch.from_numpy(r.points).to(dev) for r in same]

    def replay_same(server):
        reqs = [serving.Request(i, 0.0, c) for i, c in enumerate(same_dev)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        server.run(reqs)
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    replay_same(srv)
    same_served = min(replay_same(srv) for _ in range(3))
    tune = sorted({ln for c in [srv.ctx] + srv.worker_ctx for ln in c.autotune_log().splitlines()})
    srv.close()
    # the per-call drop-in on the same stream
    p_walls, p_outs = [], []
    plain_build_s = None
    same_plain = None
    plain_stats = {}
    if not args.skip_plain:
        plain = serving.PlainServer(device=local, solve_maxit=SOLVE_MAXIT)
        replay(plain, on_dev)
        for _ in range(2):
            out, wall = replay(plain, on_dev)
            p_walls.append(wall)
            p_outs.extend(out)
        same_plain = min(replay_same(plain) for _ in range(2))
        # per-kernel device times of the per-call path: one request at a time,
        # so every launch has the GPU to itself (the served replay's times
        # include waiting for SMs that other requests' kernels hold)
        plain.ctx.profile(True)
        replay(plain, on_dev)
        plain_stats = plain.ctx.profile_stats()
        plain.ctx.profile(False)
        plain.close()
        plain_build_s = sum(r.t_built - r.t_admit for r in p_outs) / 2
    # build + balance requests only (the served-vs-plain figure for
    # construction and balance), on the same clouds: with the stream's
    # Poisson arrivals, and as a burst (every request waiting at the start,
    # the servers' capacity)
    def replay_build(server, burst):
        reqs = [serving.Request(r.rid, 0.0 if burst else r.arrival, c) for r, c in zip(host, on_dev)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = server.run(reqs)
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    build_only = {}
    sb = serving.BatchingServer(device=local, workers=1, solve=False)
    pb = serving.PlainServer(device=local, solve=False)
    for mode in ("poisson", "burst"):
        row = {}
        for name, server in (("served", sb), ("plain", pb)):
            replay_build(server, mode == "burst")
            runs = [replay_build(server, mode == "burst") for _ in range(3)]
            out_b, wall_b = min(runs, key=lambda t: t[1])
            row[name] = {"Mpts_per_s": npts / wall_b / 1e6, **_latency(out_b)}
        row["served_over_plain"] = row["served"]["Mpts_per_s"] / row["plain"]["Mpts_per_s"]
        build_only[mode] = row
    sb.close()
    pb.close()
    errors = sum(1 for r in outs + p_outs if r.error)
    ms = 1e3 * sum(walls) / len(walls)
    res = {
        "ms_per_step": ms,
        "points": npts,
        "requests": len(host),
        "value": npts / (ms * 1e-3) / 1e6,
        "e2e_ms": 1e3 * sum(e2e_walls) / len(e2e_walls) if e2e_walls else float("nan"),
        "served": {"Mpts_per_s": npts / (ms * 1e-3) / 1e6, **_latency(outs),
                   "mean_batch": float(np.mean(batches)) if batches else None},
        "plain": ({"Mpts_per_s": npts / (sum(p_walls) / len(p_walls)) / 1e6, **_latency(p_outs)} if p_walls
                  else None),
        "iterations_max": max(r.iterations for r in outs),
        "relres_max": max(r.relres for r in outs),
        "errors": errors,
        "d2h_bytes_per_step": d2h,
        "plain_stats": plain_stats,
        "build_balance_only": build_only,
        "served_same_sample": {"requests": len(same), "points": same_pts,
                               "served_Mpts_per_s": same_pts / same_served / 1e6,
                               "plain_Mpts_per_s": (same_pts / same_plain / 1e6) if same_plain else None,
                               "note": "the reference arm's sample (all requests at once), served on the GPU"},
        "stats": stats,
        "clocks": clocks,
        "autotune": tune,
    }
    res["served_over_plain"] = (res["served"]["Mpts_per_s"] / res["plain"]["Mpts_per_s"]) if p_walls else None
    # the construction + balance phase alone: the batches' build time inside
    # the stream (sharing the GPU with the other requests' solves) against the
    # per-call builds of the plain server (which have the GPU to themselves);
    # the batching block measures batched vs per-call builds without contention
    res["build_balance"] = {"served_Mpts_per_s": npts / served_build_s / 1e6 if served_build_s else None,
                            "plain_Mpts_per_s": npts / plain_build_s / 1e6 if plain_build_s else None}
    if served_build_s and plain_build_s:
        res["build_balance"]["served_over_plain"] = plain_build_s / served_build_s
    return res


def run_scale(args, dg, ctx, local):
    """64e6 log-normal points: build+balance Mpts/s (device and host
    buffers), per-kernel figures, mesh build, FP32 / FP64 matVec."""
    import torch

    from dendro_gb300 import datagen

    npts = args.scale_npts
    host = datagen.lognormal(npts, seed=0)
    pinned = torch.from_numpy(host).pin_memory()
    dev = pinned.to(f"cuda:{local}")
    torch.cuda.synchronize()

    def step():
        lin = dg.points2Octree(dev, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
        bal = dg.balanceOctree(lin)
        n_lin, n_bal = lin.size, bal.size
        lin.free()
        return bal, n_lin, n_bal

    for _ in range(3):
        bal, n_lin, n_bal = step()
        bal.free()
    ctx.profile(True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    e0.record()
    t0 = time.perf_counter()
    for _ in range(reps):
        bal, n_lin, n_bal = step()
        bal.free()
    e1.record()
    torch.cuda.synchronize()
    ms = max(e0.elapsed_time(e1), 1e3 * (time.perf_counter() - t0)) / reps
    stats = ctx.profile_stats()
    ctx.profile(False)
    out_host = torch.empty((n_bal, 4), dtype=torch.int32).pin_memory()
    e2e = []
    for i in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lin = dg.points2Octree(pinned.numpy(), maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
        bal = dg.balanceOctree(lin)
        lin.free()
        bal.download_to(out_host.numpy())
        bal.free()
        if i > 0:
            e2e.append(time.perf_counter() - t0)
    peak, _ = _peaks()
    kernels = {k: {"ms_per_step": v[0] / reps, "launches_per_step": v[1] / reps,
                   "GB/s": (v[2] / (v[0] * 1e-3) / 1e9) if v[0] > 0 else None}
               for k, v in sorted(stats.items(), key=lambda kv: -kv[1][0])[:12]}
    top, (tms, tcnt, tbytes) = max(stats.items(), key=lambda kv: kv[1][0])
    # the step's algorithmic bytes: 40 per point to form its key (24 read,
    # 16 written), 32 per key to sort it and 32 to drop duplicates (16 read,
    # 16 written), 32 per constructed octant and 32 per balanced octant
    step_bytes = 104.0 * npts + 32.0 * n_lin + 32.0 * n_bal
    res = {"workload": "lognormal64m", "points": npts, "octants_p2o": n_lin, "octants_balanced": n_bal,
           "build_balance_Mpts_per_s": npts / (ms * 1e-3) / 1e6, "ms_per_step": ms,
           "step_algorithmic_bytes": step_bytes, "step_algorithmic_GB_per_s": step_bytes / (ms * 1e-3) / 1e9,
           "step_frac_of_measured_peak": step_bytes / (ms * 1e-3) / 1e9 / peak,
           "e2e_Mpts_per_s": npts / (sum(e2e) / len(e2e)) / 1e6,
           "top_kernel": {"name": top, "ms_per_launch": tms / tcnt, "GB/s": tbytes / (tms * 1e-3) / 1e9,
                          "frac_of_measured_peak": tbytes / (tms * 1e-3) / 1e9 / peak,
                          "traffic_per_launch": (TRAFFIC_PER_ALG_BYTE[top] * tbytes / tcnt
                                                 if top in TRAFFIC_PER_ALG_BYTE else None)},
           "kernels": kernels, "autotune": ctx.autotune_log().splitlines()}
    if not args.skip_da:
        lin = dg.points2Octree(dev, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
        bal = dg.balanceOctree(lin)
        lin.free()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        da = dg.DA(bal)
        res["da_build_ms"] = 1e3 * (time.perf_counter() - t0)
        ctx.profile(True)  # a second build, timed per kernel
        dg.DA(bal).free()
        res["da_kernels_ms"] = _top_kernels(ctx.profile_stats())
        ctx.profile(False)
        bal.free()
        V, E = da.n_node, da.n_elem
        res["n_elem"], res["n_node"] = E, V
        mv = {}
        # fp32 / fp64: the run form of the element loop (default); *_pairs: its pair form
        for name, prec, dt, form in (("fp32", 32, torch.float32, "runs"), ("fp32_pairs", 32, torch.float32, "pairs"),
                                     ("fp64", 64, torch.float64, "runs"), ("fp64_pairs", 64, torch.float64, "pairs")):
            ctx.set_matvec_form(form)
            x = torch.rand(V, dtype=dt, device=f"cuda:{local}") * 2 - 1
            y = torch.empty_like(x)
            for _ in range(3):
                da.matvec(x, y, precision=prec)
            ctx.profile(True)
            for _ in range(10):
                da.matvec(x, y, precision=prec)
            st = ctx.profile_stats()[f"matvec_fp{prec}"]
            ctx.profile(False)
            kms = st[0] / st[1]
            nbytes = 36 * E + 3 * (prec // 8) * V
            mv[name] = {"ms": kms, "GB/s": nbytes / (kms * 1e-3) / 1e9,
                        "frac_of_measured_peak": nbytes / (kms * 1e-3) / 1e9 / peak, "algorithmic_bytes": nbytes}
        ctx.set_matvec_form("runs")
        # FP32 against FP64 on the same input: relative L2 difference
        x64 = torch.rand(V, dtype=torch.float64, device=f"cuda:{local}") * 2 - 1
        y64, y32 = torch.empty_like(x64), torch.empty(V, dtype=torch.float32, device=f"cuda:{local}")
        da.matvec(x64, y64, precision=64)
        da.matvec(x64.float(), y32, precision=32)
        mv["fp32_vs_fp64_rel_l2"] = float(torch.linalg.vector_norm(y32.double() - y64) / torch.linalg.vector_norm(y64))
        res["matvec"] = mv
        da.free()
    del dev, pinned
    torch.cuda.empty_cache()
    return res


def run_batching(args, dg, ctx, local):
    """256 Gaussian-mixture clouds: one segmented points2Octree +
    balanceOctree over all of them vs one call pair per cloud."""
    import numpy as np
    import torch

    from dendro_gb300 import datagen

    clouds = datagen.batch_clouds(args.batch_clouds)
    sizes = np.array([len(c) for c in clouds], np.int64)
    seg = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    dev = torch.from_numpy(np.concatenate(clouds)).to(f"cuda:{local}")
    del clouds
    npts = int(seg[-1])
    torch.cuda.synchronize()

    def batched():
        lin = dg.points2OctreeBatch(dev, seg_start=seg, ctx=ctx)
        bal = dg.balanceOctree(lin)
        lin.free()
        off = bal.segments()
        bal.free()
        return off

    def per_call():
        counts = []
        for s in range(len(sizes)):
            lin = dg.points2Octree(dev[int(seg[s]):int(seg[s + 1])], maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
            bal = dg.balanceOctree(lin)
            lin.free()
            counts.append(bal.size)
            bal.free()
        return counts

    for _ in range(2):
        off = batched()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        off = batched()
    torch.cuda.synchronize()
    t_b = (time.perf_counter() - t0) / reps
    counts = per_call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    counts = per_call()
    torch.cuda.synchronize()
    t_p = time.perf_counter() - t0
    same = bool(np.array_equal(np.diff(np.asarray(off, np.int64)), np.asarray(counts, np.int64)))
    del dev
    torch.cuda.empty_cache()
    return {"clouds": len(sizes), "points": npts, "balanced_octants": int(off[-1]),
            "batched_Mpts_per_s": npts / t_b / 1e6, "per_call_Mpts_per_s": npts / t_p / 1e6,
            "batched_over_per_call": t_p / t_b, "batched_ms": 1e3 * t_b, "per_call_ms": 1e3 * t_p,
            "per_cloud_sizes_equal": same}


def run_poisson(args, dg, ctx, local):
    """-lap(u) + u = f, u = 0 on the cube boundary, on the balanced octree of
    16e6 N(0.5, 0.15^2) points (seed 3), f = 4 Gaussian bumps (seed 3), load
    vector = mass matrix times nodal f; levels by coarsen + balance down to
    <= 4096 elements; CG to 1e-8 relative residual with one V(2,2) damped-
    Jacobi (omega 0.667) cycle per iteration, FP32 or FP64 cycle, FP64 CG."""
    import torch

    from dendro_gb300 import datagen

    npts = args.poisson_npts
    pts = torch.from_numpy(datagen.gaussian(npts, 0.5, 0.15, seed=3)).to(f"cuda:{local}")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lin = dg.points2Octree(pts, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
    bal = dg.balanceOctree(lin)
    lin.free()
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    dg.MultiGrid(bal, max_coarse_elems=4096, ctx=ctx).free()  # loads the set-up's kernels
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mg = dg.MultiGrid(bal, max_coarse_elems=4096, ctx=ctx)
    t_setup = time.perf_counter() - t0
    ctx.profile(True)  # a second set-up, timed per kernel
    dg.MultiGrid(bal, max_coarse_elems=4096, ctx=ctx).free()
    setup_kernels = _top_kernels(ctx.profile_stats(), 20)
    ctx.profile(False)
    bal.free()
    f = datagen.bumps(mg.level_nodes(0, device=True))
    torch.cuda.synchronize()
    b = mg.rhs(f)
    out = {"points": npts, "levels": mg.n_levels, "level_elements": [e for e, _ in mg.sizes],
           "fine_nodes": mg.sizes[0][1], "build_balance_ms": 1e3 * t_build, "mg_setup_ms": 1e3 * t_setup,
           "mg_setup_kernels_ms": setup_kernels}
    xs = {}
    # fp32_vcycle: FP32 V-cycle, double-single CG operator (the default);
    # fp32_vcycle_fp64op: FP32 V-cycle, FP64 CG operator; fp32_vcycle_fp32op:
    # FP32 V-cycle and FP32 CG operator with FP64 residual replacement;
    # fp64_vcycle: all FP64
    for name, prec, op in (("fp32_vcycle", 32, 48), ("fp32_vcycle_fp64op", 32, 64), ("fp32_vcycle_fp32op", 32, 32),
                           ("fp64_vcycle", 64, 64)):
        mg.set_cg_operator(op)
        mg.solve(b, precision=prec, rtol=1e-8, maxit=200)  # warm-up
        times, its, rrs = [], [], []
        for _ in range(args.poisson_reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            x, it, rr = mg.solve(b, precision=prec, rtol=1e-8, maxit=200)
            torch.cuda.synchronize()
            times.append(1e3 * (time.perf_counter() - t0))
            its.append(it)
            rrs.append(rr)
        xs[name] = x
        out[name] = {"solve_ms": min(times), "iterations": its[0], "relres_fp64": max(rrs)}
        ctx.profile(True)  # one more solve, timed per kernel
        mg.solve(b, precision=prec, rtol=1e-8, maxit=200)
        out[name]["kernels_ms"] = _top_kernels(ctx.profile_stats())
        ctx.profile(False)
    mg.set_cg_operator(48)
    ref = torch.linalg.vector_norm(xs["fp64_vcycle"])
    out["fp32_vs_fp64_solution_rel_l2"] = float(torch.linalg.vector_norm(xs["fp32_vcycle"] - xs["fp64_vcycle"]) / ref)
    out["fp32op_vs_fp64_solution_rel_l2"] = float(
        torch.linalg.vector_norm(xs["fp32_vcycle_fp32op"] - xs["fp64_vcycle"]) / ref)
    out["fp64op_vs_fp64_solution_rel_l2"] = float(
        torch.linalg.vector_norm(xs["fp32_vcycle_fp64op"] - xs["fp64_vcycle"]) / ref)
    out["speedup_fp32_vs_fp64"] = out["fp64_vcycle"]["solve_ms"] / out["fp32_vcycle"]["solve_ms"]
    out["speedup_fp64op_vs_fp64"] = out["fp64_vcycle"]["solve_ms"] / out["fp32_vcycle_fp64op"]["solve_ms"]
    out["speedup_fp32op_vs_fp64"] = out["fp64_vcycle"]["solve_ms"] / out["fp32_vcycle_fp32op"]["solve_ms"]
    mg.free()
    return out


def run_rows(args, dg, ctx, local):
    """The rows beside the hot path on one log-normal cloud (--rows-npts
    points, device resident): completeOctree of a shuffled third of its
    balanced octree, Hilbert-ordered vs Morton-ordered record downloads, the
    assembled K + M (CSR) with its SpMV against the matrix-free matVec, and
    the compressed DA's memory and matVec.  Every library call returns with
    its results complete, so host clocks around a call time its device work
    and launch overhead; best of --rows-reps."""
    import torch

    from dendro_gb300 import datagen

    dev = f"cuda:{local}"
    reps = args.rows_reps

    def best(fn):
        fn()
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = fn()
            torch.cuda.synchronize()
            ts.append(1e3 * (time.perf_counter() - t0))
            if hasattr(r, "free"):
                r.free()
        return min(ts)

    pts = torch.from_numpy(datagen.lognormal(args.rows_npts, seed=5)).to(dev)
    lin = dg.points2Octree(pts, ctx=ctx)
    bal = dg.balanceOctree(lin)
    lin.free()
    del pts
    n = bal.size
    rec = torch.empty((n, 4), dtype=torch.int32, device=dev)
    res = {"workload": f"lognormal{args.rows_npts // 1_000_000}m", "points": args.rows_npts, "octants": n}

    # completeOctree (construct.cpp:518) of every third octant, shuffled
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    bal.download_to(rec)
    sub = rec[::3][torch.randperm((n + 2) // 3, device=dev, generator=g)].contiguous()
    out = dg.completeOctree(sub, 30, ctx=ctx)
    ms = best(lambda: dg.completeOctree(sub, 30, ctx=ctx))
    peak, _ = _peaks()
    io_bytes = 16.0 * (sub.shape[0] + out.size)  # records in + records out
    res["complete_octree"] = {"input_octants": sub.shape[0], "output_octants": out.size, "ms": ms,
                              "Mocts_per_s": sub.shape[0] / (ms * 1e-3) / 1e6,
                              "record_GB_per_s": io_bytes / (ms * 1e-3) / 1e9,
                              "frac_of_measured_peak": io_bytes / (ms * 1e-3) / 1e9 / peak}
    out.free()
    del sub

    # record order at the boundary
    ms_m = best(lambda: bal.download_to(rec))
    ctx.set_order("hilbert")
    ms_h = best(lambda: bal.download_to(rec))
    ctx.set_order("morton")
    res["records_download"] = {"morton_ms": ms_m, "hilbert_ms": ms_h,
                               "hilbert_Mocts_per_s": n / (ms_h * 1e-3) / 1e6,
                               "morton_GB_per_s": 32.0 * n / (ms_m * 1e-3) / 1e9}
    del rec

    # assembled K + M (odaJac.C:470) and SpMV vs the matrix-free element loop
    da = dg.DA(bal)
    csr = da.assemble()
    ms_a = best(lambda: da.assemble())
    x = torch.rand(da.n_node, dtype=torch.float64, device=dev)
    y = torch.empty_like(x)
    ms_spmv = best(lambda: csr.spmv(x, y))
    ms_mv = best(lambda: da.matvec(x, y))
    spmv_bytes = 12.0 * csr.nnz + 8.0 * (csr.n_rows + 1) + 16.0 * csr.n_rows  # A; x read and y written once
    res["assembly"] = {"n_elem": da.n_elem, "n_rows": csr.n_rows, "nnz": csr.nnz, "max_row_len": csr.max_row_len,
                       "assemble_ms": ms_a, "spmv_fp64_ms": ms_spmv, "matvec_fp64_ms": ms_mv,
                       "csr_bytes_per_row": (12 * csr.nnz + 8 * (csr.n_rows + 1)) / csr.n_rows,
                       "spmv_GB_per_s": spmv_bytes / (ms_spmv * 1e-3) / 1e9,
                       "spmv_frac_of_measured_peak": spmv_bytes / (ms_spmv * 1e-3) / 1e9 / peak}
    csr.free()

    # compressed DA (compressLut)
    dac = dg.DA(bal, compressLut=True)
    x32 = x.float()
    y32 = torch.empty_like(x32)
    res["compressed_da"] = {
        "plain_bytes_per_elem": da.memory_bytes() / da.n_elem,
        "compressed_bytes_per_elem": dac.memory_bytes() / dac.n_elem,
        "matvec_fp32_ms_plain": best(lambda: da.matvec(x32, y32, precision=32)),
        "matvec_fp32_ms_compressed": best(lambda: dac.matvec(x32, y32, precision=32)),
    }
    da.free()
    dac.free()
    bal.free()
    torch.cuda.empty_cache()
    return res


def run_ours(args):
    import torch

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()

    # the CPU baseline first: its worker processes start before this process
    # touches the GPU
    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu:
        try:
            cpu = cpu_baseline_sample(os.cpu_count() or 1)
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "Mpts/s", "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {exc}"}

    torch.cuda.set_device(local)
    import dendro_gb300 as dg

    ctx = dg.Context(local)
    if args.skip_serve:  # profiling runs of the other blocks only
        extra = {}
        if not args.skip_scale:
            extra["scale"] = run_scale(args, dg, ctx, local)
        if not args.skip_batch:
            extra["batching"] = run_batching(args, dg, ctx, local)
        if not args.skip_mg:
            extra["precision"] = run_poisson(args, dg, ctx, local)
        if not args.skip_rows:
            extra["next_rows"] = run_rows(args, dg, ctx, local)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": None, "note": "serving skipped", **extra}), flush=True)
        return
    serve = run_serving(args, local, barrier)
    ms = serve["ms_per_step"]
    e2e_ms = serve["e2e_ms"]
    if ws > 1:
        ms, e2e_ms = max_over_ranks([ms, e2e_ms], f"cuda:{local}")
    value = replica_value(ws, serve["points"], ms)
    extra = {}
    if not args.skip_scale:
        extra["scale"] = run_scale(args, dg, ctx, local)
    if not args.skip_batch:
        extra["batching"] = run_batching(args, dg, ctx, local)
    if not args.skip_mg:
        extra["precision"] = run_poisson(args, dg, ctx, local)
    if not args.skip_rows:
        extra["next_rows"] = run_rows(args, dg, ctx, local)

    # roofline of the dominant kernel of the served step
    stats = serve["stats"]
    peak, peak_kind = _peaks()
    launches = sum(v[1] for v in stats.values()) * args.steps  # per step (the profiled replay) x timed steps
    tname, (tms, tcnt, tbytes) = max(stats.items(), key=lambda kv: kv[1][0])
    per_launch_ms, per_launch_bytes = tms / tcnt, tbytes / tcnt
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9
    step_total = sum(v[0] for v in stats.values())
    # stats hold one profiled replay of the step
    kernels = {k: {"ms_per_step": v[0], "launches_per_step": v[1],
                   "GB/s": (v[2] / (v[0] * 1e-3) / 1e9) if v[0] > 0 else None,
                   "share": v[0] / step_total if step_total else None}
               for k, v in sorted(stats.items(), key=lambda kv: -kv[1][0])[:15]}
    # the same figures from the per-call path's profiled replay (sequential)
    pst = serve["plain_stats"]
    roof_seq, kernels_seq = None, None
    if pst and tname in pst:
        sms, scnt, sbytes = pst[tname]
        sach = (sbytes / scnt) / (sms / scnt * 1e-3) / 1e9
        roof_seq = {"kernel": tname, "achieved": sach, "peak": peak, "unit": "GB/s", "frac": sach / peak,
                    "ms_per_launch": sms / scnt, "algorithmic_bytes_per_launch": sbytes / scnt,
                    "note": "per-call path, one request at a time: each launch has the GPU to itself"}
        ptot = sum(v[0] for v in pst.values())
        kernels_seq = {k: {"ms": v[0], "launches": v[1], "share": v[0] / ptot}
                       for k, v in sorted(pst.items(), key=lambda kv: -kv[1][0])[:15]}
    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "Mpts/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "int keys (octree, mesh); FP32 V-cycle, FP64 CG vectors with a double-single operator (solve)",
            "data": "synthetic",
            "config": {"workload": "serving stream", "requests": serve["requests"], "points": serve["points"],
                       "rate_req_s": SERVE_RATE, "sizes": list(SERVE_SIZES), "seed": SERVE_SEED,
                       "max_depth": 30, "max_pts_per_octant": 1, "solve": f"FP32 V(2,2) CG (double-single operator, FP64 vectors) to 1e-8, <= {SOLVE_MAXIT} it",
                       "parallelism": f"replicas x{ws}",
                       "l2": f"inputs larger than L2 ({24 * serve['points'] / 1e9:.2f} GB of points per step)"},
            "autotune": serve["autotune"],
            "served": serve["served"],
            "plain": serve["plain"],
            "served_over_plain": serve["served_over_plain"],
            "build_balance_in_stream": {**serve["build_balance"],
                                        "note": "served builds share the GPU with solves; see batching"},
            "solve_iterations_max": serve["iterations_max"],
            "solve_relres_max": serve["relres_max"],
            "request_errors": serve["errors"],
            "e2e": {"value": replica_value(ws, serve["points"], e2e_ms), "unit": "Mpts/s",
                    "h2d_bytes_per_step": 24 * serve["points"], "d2h_bytes_per_step": serve["d2h_bytes_per_step"],
                    "d2h": "each request's FP64 solution vector, into pinned host memory"},
            "served_same_sample": serve["served_same_sample"],
            "serving_build_balance": {**serve["build_balance_only"],
                                      "note": ("requests of build + balance only, same clouds; burst = every "
                                               "request waiting at the start")},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": tname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": (TRAFFIC_PER_ALG_BYTE[tname] * per_launch_bytes
                                     if tname in TRAFFIC_PER_ALG_BYTE else None),
                         "traffic_source": ("ncu capture of a smaller launch, scaled by algorithmic bytes"
                                            if tname in TRAFFIC_PER_ALG_BYTE else None),
                         "algorithmic_bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_ms},
            "clocks": serve["clocks"],
            "cpu_baseline": cpu,
            "kernels": kernels,
            "roofline_sequential": roof_seq,
            "kernels_per_call": kernels_seq,
            "kernels_note": ("device ms of one replay of the step with each launch timed by CUDA events on its "
                             "stream (the timed steps replay the CG iterations from CUDA graphs instead)"),
            **extra,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--serve-requests", type=int, default=SERVE_REQUESTS)
    ap.add_argument("--serve-workers", type=int, default=8, help="solver streams of the batching server")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--scale-npts", type=int, default=64_000_000)
    ap.add_argument("--batch-clouds", type=int, default=256)
    ap.add_argument("--poisson-npts", type=int, default=16_000_000)
    ap.add_argument("--poisson-reps", type=int, default=3)
    ap.add_argument("--skip-scale", action="store_true")
    ap.add_argument("--skip-da", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--skip-mg", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-rows", action="store_true")
    ap.add_argument("--rows-npts", type=int, default=8_000_000)
    ap.add_argument("--rows-reps", type=int, default=3)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
