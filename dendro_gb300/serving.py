"""Serving of octree + Poisson requests on one GPU, with continuous batching.

A request carries one point cloud.  Its work is the full request of the serving workload:
points2Octree -> balanceOctree -> mesh -> multigrid set-up -> CG with an
FP32 V-cycle (FP64 residuals), at most ``solve_maxit`` iterations; with
``solve=False`` a request is points2Octree -> balanceOctree only.

``PlainServer`` is the per-call drop-in: one request at a time, in arrival
order, every call made for that cloud alone.

``BatchingServer`` is continuous batching:
  * admission: a request enters the device only while the estimated HBM
    bytes of everything in flight stay under ``hbm_budget`` (estimate from
    the point count, ``estimate_bytes``); others wait in arrival order;
  * build: every admitted request not yet built joins the next batch, and
    the whole batch goes through ONE segmented points2Octree +
    balanceOctree (points2OctreeBatch): requests that arrive while a batch
    is on the GPU form the next batch as soon as it completes;
  * solve: each cloud's octree is extracted and handed to a pool of solver
    workers, each with its own CUDA stream (dg_ctx), so solves of different
    requests overlap on the device and with the next batch's build.
Results are identical to the plain path's (tests/test_gpu_serving.py).
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import datagen
from .api import Context, MultiGrid, balanceOctree, points2Octree, points2OctreeBatch


@dataclass
class Request:
    rid: int
    arrival: float            # seconds from the start of the stream
    points: np.ndarray        # (n, 3) float64
    t_admit: float = 0.0
    t_built: float = 0.0
    t_done: float = 0.0
    n_octants: int = 0
    n_balanced: int = 0
    iterations: int = 0
    relres: float = 0.0
    solution_norm: float = 0.0
    t_setup: float = 0.0        # multigrid set-up seconds (mesh hierarchy)
    error: str = ""
    # results handed back to the caller (filled when the server keeps them):
    # the balanced octree's {x, y, z, level} records, and the FP64 solution
    # with the coordinates of its nodes (level-0 numbering of the request)
    octree: np.ndarray | None = None
    solution: np.ndarray | None = None
    node_xyz: np.ndarray | None = None

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


def estimate_bytes(npts: int) -> int:
    """HBM bytes one request holds at its peak: points (24 B), construction
    keys (~3.4 octants/pt x 16 B x 2), balanced octree (~5.6/pt x 16 B),
    mesh (~5.6 elements/pt x 40 B) and the multigrid hierarchy and vectors
    (~5.6 x 80 B); rounded up."""
    return int(npts * (24 + 3.4 * 32 + 5.6 * 16 + 5.6 * 40 + 5.6 * 80)) + (64 << 20)


def admit(waiting: list, in_flight: int, budget: int, max_batch_points: int):
    """The next batch from the head of ``waiting`` (removed from it, in
    arrival order): requests join while the estimated bytes in flight stay
    within ``budget`` and the batch within ``max_batch_points`` points; a
    request that alone exceeds the budget is admitted when nothing else is in
    flight.  Returns ([(request, bytes)], new bytes in flight)."""
    batch, npts = [], 0
    while waiting:
        n = len(waiting[0].points)
        need = estimate_bytes(n)
        fits = in_flight + need <= budget or (not batch and in_flight == 0)
        if not fits or (batch and npts + n > max_batch_points):
            break
        batch.append((waiting.pop(0), need))
        in_flight += need
        npts += n
    return batch, in_flight


def poisson_stream(count: int, rate: float = 200.0, lo: float = 1e4, hi: float = 8e6, seed: int = 4) -> list:
    """Poisson arrivals (mean ``rate``/s), sizes log-uniform in [lo, hi],
    half Gaussian-mixture clouds and half log-normal clouds."""
    rng = np.random.Generator(np.random.PCG64(seed))
    gaps = rng.exponential(1.0 / rate, count)
    sizes = np.round(datagen._exp(rng.uniform(datagen._ln(lo), datagen._ln(hi), count))).astype(np.int64)
    reqs = []
    t = 0.0
    for i in range(count):
        t += gaps[i]
        if i % 2 == 0:
            pts = datagen.mixture(int(sizes[i]), rng)
        else:
            pts = datagen.lognormal(int(sizes[i]), seed=int(rng.integers(1 << 30)))
        reqs.append(Request(i, t, pts))
    return reqs


def _solve(ctx: Context, bal, req: Request, maxit: int, max_coarse: int, stream=None, keep: str = ""):
    """Mesh + multigrid + FP32-V-cycle CG for one balanced octree, all on the
    device: the right-hand side field is evaluated at the device-resident
    node coordinates.  The iteration count, the residual and the solution
    norm always come back to the host; ``keep`` names what else does:
    "solution" (the FP64 solution vector, into pinned host memory) and
    "octree" (the balanced octree records and the node coordinates).
    ``stream``: the torch stream for the field evaluation (synchronised
    before the library reads it)."""
    import torch

    t0 = time.perf_counter()
    if "octree" in keep:
        req.octree = bal.to_numpy(ctx)
    mg = MultiGrid(bal, max_coarse_elems=max_coarse, ctx=ctx)
    try:
        req.t_setup = time.perf_counter() - t0
        with torch.cuda.stream(stream or torch.cuda.current_stream(ctx.device)):
            nodes = mg.level_nodes(0, device=True)
            f = datagen.bumps(nodes)
            torch.cuda.current_stream(ctx.device).synchronize()
        b = mg.rhs(f)
        x, it, rr = mg.solve(b, precision=32, rtol=1e-8, maxit=maxit)
        req.iterations, req.relres = it, rr
        with torch.cuda.stream(stream or torch.cuda.current_stream(ctx.device)):
            req.solution_norm = float(torch.linalg.vector_norm(x))
            if "solution" in keep:
                host = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
                host.copy_(x, non_blocking=True)
            if "octree" in keep:
                req.node_xyz = nodes.cpu().numpy().view(np.uint32)
            torch.cuda.current_stream(ctx.device).synchronize()
            if "solution" in keep:
                req.solution = host.numpy()
    finally:
        mg.free()


def _host_or_device(points):
    """Points as the API takes them: a numpy array (host, pinned or not) or a
    CUDA tensor; a CPU tensor is passed as its numpy view (same memory)."""
    if hasattr(points, "is_cuda") and not points.is_cuda:
        return points.numpy()
    return points


class PlainServer:
    """One request at a time through the single-cloud API."""

    def __init__(self, device: int = 0, solve_maxit: int = 50, max_coarse: int = 4096, keep: str = "",
                 solve: bool = True):
        self.ctx = Context(device)
        self.maxit, self.max_coarse = solve_maxit, max_coarse
        self.keep = keep  # results copied back per request (see _solve)
        self.solve = solve  # False: a request is points2Octree + balanceOctree only

    def run(self, reqs: list) -> list:
        t0 = time.perf_counter()
        for r in sorted(reqs, key=lambda q: q.arrival):
            now = time.perf_counter() - t0
            if now < r.arrival:
                time.sleep(r.arrival - now)
            r.t_admit = time.perf_counter() - t0
            lin = points2Octree(_host_or_device(r.points), ctx=self.ctx)
            bal = balanceOctree(lin)
            r.n_octants, r.n_balanced = lin.size, bal.size
            lin.free()
            r.t_built = time.perf_counter() - t0
            if not self.solve:
                if "octree" in self.keep:
                    r.octree = bal.to_numpy()
            else:
                try:
                    _solve(self.ctx, bal, r, self.maxit, self.max_coarse, keep=self.keep)
                except Exception as e:  # reported per request
                    r.error = str(e)
            bal.free()
            r.t_done = time.perf_counter() - t0
        return reqs

    def close(self):
        self.ctx.close()


class BatchingServer:
    """Continuous batching: admission by HBM budget, one segmented
    construction + balance per batch, solves overlapped on worker streams."""

    def __init__(self, device: int = 0, hbm_budget: int = 64 << 30, workers: int = 3, solve_maxit: int = 50,
                 max_coarse: int = 4096, max_batch_points: int = 64_000_000, keep: str = "", solve: bool = True):
        self.keep = keep  # results copied back per request (see _solve)
        self.solve = solve  # False: a request is points2Octree + balanceOctree only
        self.ctx = Context(device)
        self.worker_ctx = [Context(device) for _ in range(workers)]
        self.budget, self.maxit, self.max_coarse = hbm_budget, solve_maxit, max_coarse
        self.max_batch_points = max_batch_points
        self.in_flight = 0
        self.cv = threading.Condition()
        self.batches = []  # sizes of the batches that were built
        self.build_s = []  # seconds of each batch's construction + balance

    def _release(self, nbytes: int):
        with self.cv:
            self.in_flight -= nbytes
            self.cv.notify_all()

    def _worker(self, ctx: Context, work: queue.Queue, t0: float):
        import torch

        stream = torch.cuda.Stream(device=ctx.device)
        while True:
            item = work.get()
            if item is None:
                return
            req, bal, nbytes = item
            try:
                _solve(ctx, bal, req, self.maxit, self.max_coarse, stream, keep=self.keep)
            except Exception as e:  # reported per request
                req.error = str(e)
            finally:
                bal.free(ctx)
                req.t_done = time.perf_counter() - t0
                self._release(nbytes)

    def run(self, reqs: list) -> list:
        reqs = sorted(reqs, key=lambda q: q.arrival)
        arrived: queue.Queue = queue.Queue()
        work: queue.Queue = queue.Queue()
        t0 = time.perf_counter()

        def arrivals():
            for r in reqs:
                now = time.perf_counter() - t0
                if now < r.arrival:
                    time.sleep(r.arrival - now)
                arrived.put(r)
            arrived.put(None)

        producers = [threading.Thread(target=arrivals, daemon=True)]
        workers = [threading.Thread(target=self._worker, args=(c, work, t0), daemon=True) for c in self.worker_ctx]
        for t in producers + workers:
            t.start()
        waiting, done_arriving = [], False
        while True:
            # everything that has arrived so far joins the waiting line
            block = not waiting and not done_arriving
            while True:
                try:
                    r = arrived.get(block=block, timeout=None)
                except queue.Empty:
                    break
                block = False
                if r is None:
                    done_arriving = True
                    break
                waiting.append(r)
            if not waiting:
                if done_arriving:
                    break
                continue
            # admission by the HBM budget, in arrival order
            with self.cv:
                batch, self.in_flight = admit(waiting, self.in_flight, self.budget, self.max_batch_points)
                now = time.perf_counter() - t0
                for r, _ in batch:
                    r.t_admit = now
                if not batch:
                    self.cv.wait(timeout=0.05)
                    continue
            # one segmented construction + balance for the whole batch; host
            # clouds are copied in one by one (from pinned memory when they
            # live there) and joined on the device
            tb0 = time.perf_counter() - t0
            clouds = [r.points for r, _ in batch]
            if not all(getattr(c, "is_cuda", False) for c in clouds):
                import torch

                dev = f"cuda:{self.ctx.device}"
                clouds = [torch.as_tensor(c).to(dev, non_blocking=True) for c in clouds]
                torch.cuda.current_stream(self.ctx.device).synchronize()
            lin = points2OctreeBatch(clouds, ctx=self.ctx)
            bal = balanceOctree(lin)
            off_lin, off_bal = lin.segments(), bal.segments()
            lin.free()
            self.batches.append(len(batch))
            tb = time.perf_counter() - t0
            self.build_s.append(tb - tb0)
            for s, (r, need) in enumerate(batch):
                r.n_octants = int(off_lin[s + 1] - off_lin[s])
                r.n_balanced = int(off_bal[s + 1] - off_bal[s])
                r.t_built = tb
                if self.solve:
                    work.put((r, bal.extract(s), need))
            if not self.solve:  # build + balance requests end with the batch
                if "octree" in self.keep:
                    recs, off = bal.to_numpy(), off_bal
                    for s, (r, _) in enumerate(batch):
                        r.octree = recs[off[s]:off[s + 1]]
                done = time.perf_counter() - t0
                for r, need in batch:
                    r.t_done = done
                    self._release(need)
            bal.free()
        for _ in workers:
            work.put(None)
        for t in workers:
            t.join()
        return reqs

    def close(self):
        for c in self.worker_ctx:
            c.close()
        self.ctx.close()


def summarize(reqs: list, wall: float) -> dict:
    lat = np.array([r.latency for r in reqs]) * 1e3
    pts = sum(len(r.points) for r in reqs)
    return {
        "requests": len(reqs),
        "points": int(pts),
        "wall_s": wall,
        "Mpts_per_s": pts / wall / 1e6,
        "p50_ms": float(np.percentile(lat, 50)),
        "p99_ms": float(np.percentile(lat, 99)),
        "errors": sum(1 for r in reqs if r.error),
        "max_relres": max((r.relres for r in reqs), default=0.0),
    }
