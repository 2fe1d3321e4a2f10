"""Benchmark of the octree hot path: points2Octree + balanceOctree(incCorner).

Workload (default): 64e6 points, per axis u = exp(N(0,1)) mapped by u/(1+u)
into (0,1), FP64 coordinates, seed 0 (numpy PCG64), maxDepth 30,
maxNumPtsPerOctant 1 — the scale configuration.  One step = one
points2Octree followed by one balanceOctree of that cloud.

  value : Mpts/s with the points already resident in HBM (device-timed)
  e2e   : the same through the C ABI with host buffers: the step's points
          copied in from pinned host memory and the balanced octree copied
          back to pinned host memory, inside the timed region
Also reported: the mesh (ot::DA) build time and the Laplacian+mass matVec
(FP32 and FP64) on the balanced octree of the workload, per-kernel roofline
figures, nvidia-smi clocks sampled during the timed region, and the CPU
oracle timed on a bounded sample of the same workload.

--impl reference times the CPU restatement of the reference path (oracle/,
C) on the host cores: one process per core, each building and balancing its
own bounded sample of the workload per step.

Multi-GPU: replicas only (the path has no exchange step); each rank builds
its own copy of the workload, value sums the ranks' points over the slowest
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

WORKLOADS = {
    # name: (npts, generator description)
    "lognormal64m": 64_000_000,
    "gauss1m": 1_000_000,
}
CPU_SAMPLE_PTS = 1_000_000


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
              "clocks_event_reasons.sw_power_cap")

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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax.append(float(r[1]))
                for nm, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_sample_run(args):
    """One bounded CPU sample: oracle points2Octree + balance (runs in a worker process)."""
    npts, seed = args
    sys.path.insert(0, ROOT)
    from dendro_gb300 import datagen
    from oracle import dg_oracle

    pts = datagen.lognormal(npts, seed=seed)
    t0 = time.perf_counter()
    lin = dg_oracle.points_to_octree(pts, 30, 1)
    bal = dg_oracle.balance(lin, 30)
    return time.perf_counter() - t0, len(lin), len(bal)


def run_reference(args):
    """CPU arm: the oracle's restatement of the reference path on every host core."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import multiprocessing as mp

    from oracle import dg_oracle

    dg_oracle.build()
    cores = os.cpu_count() or 1
    npts = args.cpu_sample
    ctxmp = mp.get_context("spawn")
    times = []
    with ctxmp.Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(cpu_sample_run, [(npts, 1000 + i) for i in range(cores)])
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                times.append(dt)
    ms = 1e3 * sum(times) / len(times)
    value = cores * npts / (ms * 1e-3) / 1e6
    line = {
        "impl": "reference",
        "metric": "build+balance throughput, Mpts/s (points2Octree + balanceOctree incCorner)",
        "value": value,
        "unit": "Mpts/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32/int64 keys, FP64 coords",
        "data": "synthetic",
        "config": {"workload": args.workload, "max_depth": 30, "max_pts_per_octant": 1,
                   "sample": f"{cores} processes x {npts} log-normal pts per step (seeds 1000+)"},
        "cpu_baseline": {"value": value, "unit": "Mpts/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} x {npts} pts per step, oracle C restatement, 1 thread per process"},
        "e2e": {"value": value, "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _top_kernels(stats: dict, k: int = 10) -> dict:
    """{kernel: [total ms, launches]} of the k kernels with the most time."""
    top = sorted(stats.items(), key=lambda kv: -kv[1][0])[:k]
    return {name: [round(v[0], 3), int(v[1])] for name, v in top}


def run_poisson(dg, datagen, ctx, local, args):
    """-lap(u) + u = f, u = 0 on the cube boundary, on the balanced octree of
    16e6 N(0.5, 0.15^2) points (seed 3), f = 4 Gaussian bumps (seed 3), load
    vector = mass matrix times nodal f; levels by coarsen + balance down to
    <= 4096 elements; CG to 1e-8 relative residual with one V(2,2) damped-
    Jacobi (omega 0.667) cycle per iteration, FP32 or FP64 cycle, FP64 CG."""
    import torch

    npts = args.poisson_npts
    pts = torch.from_numpy(datagen.gaussian(npts, 0.5, 0.15, seed=3)).to(f"cuda:{local}")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lin = dg.points2Octree(pts, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
    bal = dg.balanceOctree(lin)
    lin.free()
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    mg = dg.MultiGrid(bal, max_coarse_elems=4096)
    t_setup = time.perf_counter() - t0
    bal.free()
    f = torch.from_numpy(datagen.bumps(mg.level_nodes(0))).to(f"cuda:{local}")
    b = mg.rhs(f)
    out = {"points": npts, "levels": mg.n_levels, "level_elements": [e for e, _ in mg.sizes],
           "fine_nodes": mg.sizes[0][1], "build_balance_ms": 1e3 * t_build, "mg_setup_ms": 1e3 * t_setup}
    for prec in (32, 64):
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
        out[f"fp{prec}_vcycle"] = {"solve_ms": min(times), "iterations": its[0], "relres_fp64": max(rrs)}
        ctx.profile(True)  # one more solve, timed per kernel
        mg.solve(b, precision=prec, rtol=1e-8, maxit=200)
        out[f"fp{prec}_vcycle"]["kernels_ms"] = _top_kernels(ctx.profile_stats())
        ctx.profile(False)
    out["speedup_fp32_vs_fp64"] = out["fp64_vcycle"]["solve_ms"] / out["fp32_vcycle"]["solve_ms"]
    mg.free()
    return out


def run_ours(args):
    import numpy as np
    import torch

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()

    import dendro_gb300 as dg
    from dendro_gb300 import datagen

    npts = args.npts or WORKLOADS[args.workload]
    if args.workload.startswith("lognormal"):
        host = datagen.lognormal(npts, seed=0)
    else:
        host = datagen.gaussian(npts, 0.5, 0.1, seed=0)
    pinned = torch.from_numpy(host).pin_memory()
    dev = pinned.to(f"cuda:{local}")
    ctx = dg.Context(local)
    torch.cuda.synchronize()

    def step_device():
        lin = dg.points2Octree(dev, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
        bal = dg.balanceOctree(lin)
        n_lin, n_bal = lin.size, bal.size
        lin.free()
        return bal, n_lin, n_bal

    for _ in range(args.warmup):
        bal, n_lin, n_bal = step_device()
        bal.free()
    torch.cuda.synchronize()

    # ---- device-resident timed region --------------------------------------
    ctx.profile(True)
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bal, n_lin, n_bal = step_device()
        bal.free()
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier()
    clocks = sampler.stop()
    stats = ctx.profile_stats()
    ctx.profile(False)
    ms = e0.elapsed_time(e1) / args.steps
    ms = max(ms, 1e3 * wall / args.steps)  # host waits inside the calls count too
    if ws > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * npts / (ms * 1e-3) / 1e6

    # ---- end-to-end through the C ABI with host buffers --------------------
    out_host = torch.empty((n_bal, 4), dtype=torch.int32).pin_memory()
    e2e_ms = []
    for i in range(args.steps + 1):
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lin = dg.points2Octree(pinned.numpy(), maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
        bal = dg.balanceOctree(lin)
        lin.free()
        bal.download_to(out_host.numpy())
        bal.free()
        dt = time.perf_counter() - t0
        if i > 0:
            e2e_ms.append(1e3 * dt)
    e2e_step = sum(e2e_ms) / len(e2e_ms)
    if ws > 1:
        import torch.distributed as dist

        t = torch.tensor([e2e_step], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_step = float(t.item())
    e2e = {"value": ws * npts / (e2e_step * 1e-3) / 1e6, "unit": "Mpts/s", "h2d_bytes_per_step": 24 * npts,
           "d2h_bytes_per_step": 16 * n_bal}

    # ---- mesh + matVec on the balanced octree ------------------------------
    extra = {}
    if not args.skip_da:
        lin = dg.points2Octree(dev, maxDepth=30, maxNumPtsPerOctant=1, ctx=ctx)
        bal = dg.balanceOctree(lin)
        lin.free()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        da = dg.DA(bal)
        da_ms = 1e3 * (time.perf_counter() - t0)
        ctx.profile(True)  # a second build, timed per kernel
        dg.DA(bal).free()
        da_kernels = _top_kernels(ctx.profile_stats())
        ctx.profile(False)
        bal.free()
        V, E = da.n_node, da.n_elem
        ctx.profile(True)
        mv = {}
        for prec, dt in ((32, torch.float32), (64, torch.float64)):
            x = torch.rand(V, dtype=dt, device=f"cuda:{local}") * 2 - 1
            y = torch.empty_like(x)
            for _ in range(3):
                da.matvec(x, y, precision=prec)
            ctx.profile(True)
            reps = 10
            for _ in range(reps):
                da.matvec(x, y, precision=prec)
            st = ctx.profile_stats()["matvec"]
            kms = st[0] / st[1]
            nbytes = 36 * E + 3 * (prec // 8) * V
            mv[f"fp{prec}"] = {"ms": kms, "GB/s": nbytes / (kms * 1e-3) / 1e9, "algorithmic_bytes": nbytes}
        ctx.profile(False)
        da.free()
        extra = {"da_build_ms": da_ms, "da_kernels_ms": da_kernels, "n_elem": E, "n_node": V, "matvec": mv}

    # ---- precision workload: FP32-MG vs FP64 solve to 1e-8 ----------------
    if not args.skip_mg:
        extra["poisson"] = run_poisson(dg, datagen, ctx, local, args)

    # ---- roofline of the dominant kernel of the timed step ----------------
    peak, peak_kind = _peaks()
    launches = sum(v[1] for v in stats.values())
    top = max(stats.items(), key=lambda kv: kv[1][0])
    tname, (tms, tcnt, tbytes) = top
    per_launch_ms = tms / tcnt
    per_launch_bytes = tbytes / tcnt
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9
    step_ms_total = sum(v[0] for v in stats.values())
    kernels = {k: {"ms_per_step": v[0] / args.steps, "launches_per_step": v[1] / args.steps,
                   "GB/s": (v[2] / (v[0] * 1e-3) / 1e9) if v[0] > 0 else None,
                   "share": v[0] / step_ms_total if step_ms_total else None}
               for k, v in sorted(stats.items(), key=lambda kv: -kv[1][0])}

    cpu = None
    if rank == 0 and not args.skip_cpu:
        try:
            from oracle import dg_oracle

            dg_oracle.build()
            dt, _, _ = cpu_sample_run((args.cpu_sample, 1000))
            cpu = {"value": args.cpu_sample / dt / 1e6, "unit": "Mpts/s", "cores": 1, "kind": "port",
                   "sample": f"{args.cpu_sample} log-normal pts (seed 1000), oracle C restatement of "
                             f"points2Octree + balanceOctree, 1 thread, {dt:.2f} s"}
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "Mpts/s", "cores": 1, "kind": "port", "sample": f"failed: {exc}"}

    if rank == 0:
        line = {
            "metric": "build+balance throughput, Mpts/s (points2Octree + balanceOctree incCorner)",
            "value": value,
            "unit": "Mpts/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "u64x2 Morton keys (int), FP64 coords",
            "data": "synthetic",
            "config": {"workload": args.workload, "points": npts, "max_depth": 30, "max_pts_per_octant": 1,
                       "octants_p2o": n_lin, "octants_balanced": n_bal,
                       "parallelism": f"replicas x{ws}", "l2": "inputs larger than L2 (1.5 GB of points per step)"},
            "e2e": e2e,
            "gpu_launches": int(launches // max(args.steps, 1)) * args.steps,
            "roofline": {"bound": "hbm", "kernel": tname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                         "algorithmic_bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_ms},
            "clocks": clocks,
            "cpu_baseline": cpu,
            "kernels": kernels,
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
    ap.add_argument("--workload", default="lognormal64m", choices=sorted(WORKLOADS))
    ap.add_argument("--npts", type=int, default=0, help="override the workload's point count")
    ap.add_argument("--cpu-sample", type=int, default=CPU_SAMPLE_PTS)
    ap.add_argument("--skip-da", action="store_true")
    ap.add_argument("--skip-mg", action="store_true")
    ap.add_argument("--poisson-npts", type=int, default=16_000_000)
    ap.add_argument("--poisson-reps", type=int, default=3)
    ap.add_argument("--skip-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
