"""Host API mirroring the reference's C++ entry points for the octree path.

Names and argument meaning follow Dendro4 (``ot::points2Octree``,
``ot::balanceOctree``, ``par::removeDuplicates``, ``ot::DA``,
``Jacobian1MatMult``); every call goes through the C ABI of
include/dendro_gb300.h into the CUDA library.  Arrays may be numpy arrays
(host) or CUDA tensors exposing ``data_ptr()`` (device, no copy).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import DendroError, check

__all__ = [
    "Context",
    "Octree",
    "DA",
    "DendroError",
    "points2Octree",
    "balanceOctree",
    "sortUniquePoints",
    "points2OctreeBatch",
    "coarsenOctree",
    "default_context",
]


def _is_device(a) -> bool:
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _ptr(a):
    if _is_device(a):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """One GPU, one CUDA stream (dg_ctx)."""

    def __init__(self, device: int = 0):
        self._L = _lib.load()
        h = ctypes.c_void_p()
        st = self._L.dg_ctx_create(device, ctypes.byref(h))
        if st != 0:
            raise DendroError(st, f"dg_ctx_create(device={device}): {self._L.dg_status_string(st).decode()}")
        self.handle = h
        self.device = device

    def set_stream(self, stream_ptr: int | None):
        check(self.handle, self._L.dg_ctx_set_stream(self.handle, ctypes.c_void_p(stream_ptr or 0)), "dg_ctx_set_stream")

    def last_device_ms(self) -> float:
        v = ctypes.c_double()
        self._L.dg_ctx_last_device_ms(self.handle, ctypes.byref(v))
        return v.value

    def profile(self, enable: bool = True):
        """Start (or stop) per-kernel timing; clears the statistics."""
        check(self.handle, self._L.dg_ctx_profile(self.handle, 1 if enable else 0), "dg_ctx_profile")

    def profile_stats(self) -> dict:
        """{kernel: (total_ms, launches, algorithmic_bytes)} since profile()."""
        n = ctypes.c_int()
        self._L.dg_ctx_profile_count(self.handle, ctypes.byref(n))
        out = {}
        buf = ctypes.create_string_buffer(64)
        for i in range(n.value):
            ms, cnt, b = ctypes.c_double(), ctypes.c_ulonglong(), ctypes.c_double()
            self._L.dg_ctx_profile_entry(self.handle, i, buf, 64, ctypes.byref(ms), ctypes.byref(cnt), ctypes.byref(b))
            out[buf.value.decode()] = (ms.value, cnt.value, b.value)
        return out

    def close(self):
        if getattr(self, "handle", None):
            self._L.dg_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default


class Octree:
    """Device-resident linear octree (dg_octree); records {x, y, z, level}."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self.handle = handle
        n = ctypes.c_size_t()
        d = ctypes.c_uint()
        check(ctx.handle, ctx._L.dg_octree_size(handle, ctypes.byref(n), ctypes.byref(d)), "dg_octree_size")
        self.size = n.value
        self.max_depth = d.value

    def __len__(self):
        return self.size

    def segments(self) -> np.ndarray:
        """Start offsets of each cloud's octants (nseg + 1 entries)."""
        ns = ctypes.c_size_t()
        check(self.ctx.handle, self.ctx._L.dg_octree_segments(self.ctx.handle, self.handle, ctypes.byref(ns), None),
              "dg_octree_segments")
        off = np.empty(ns.value + 1, np.uint64)
        check(self.ctx.handle, self.ctx._L.dg_octree_segments(self.ctx.handle, self.handle, ctypes.byref(ns), _ptr(off)),
              "dg_octree_segments")
        return off

    def split(self) -> list:
        """The octree of every cloud, as (n_s, 4) uint32 arrays."""
        a = self.to_numpy()
        off = self.segments()
        return [a[off[i]:off[i + 1]] for i in range(len(off) - 1)]

    def to_numpy(self) -> np.ndarray:
        out = np.empty((self.size, 4), np.uint32)
        check(self.ctx.handle, self.ctx._L.dg_octree_download(self.ctx.handle, self.handle, _ptr(out), 0), "dg_octree_download")
        return out

    def download_to(self, dst):
        """Write the records into a host array or CUDA tensor of n*4 uint32."""
        check(
            self.ctx.handle,
            self.ctx._L.dg_octree_download(self.ctx.handle, self.handle, _ptr(dst), 1 if _is_device(dst) else 0),
            "dg_octree_download",
        )

    @classmethod
    def from_numpy(cls, xyzl: np.ndarray, maxDepth: int = 30, ctx: Context | None = None) -> "Octree":
        ctx = ctx or default_context()
        a = np.ascontiguousarray(xyzl, dtype=np.uint32).reshape(-1, 4)
        h = ctypes.c_void_p()
        check(ctx.handle, ctx._L.dg_octree_upload(ctx.handle, _ptr(a), a.shape[0], maxDepth, 0, ctypes.byref(h)), "dg_octree_upload")
        return cls(ctx, h)

    def free(self):
        if self.handle:
            self.ctx._L.dg_octree_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _points_arg(pts):
    if _is_device(pts):
        if str(pts.dtype) != "torch.float64" or not pts.is_contiguous():
            raise ValueError("device points must be a contiguous float64 tensor")
        return pts, pts.numel() // 3, 1
    a = np.ascontiguousarray(pts, dtype=np.float64)
    if a.size % 3:
        raise ValueError("points must hold x, y, z triples")
    return a, a.size // 3, 0


def points2Octree(pts, gLens=(1.0, 1.0, 1.0), dim: int = 3, maxDepth: int = 30, maxNumPtsPerOctant: int = 1,
                  comm_size: int = 1, ctx: Context | None = None) -> Octree:
    """ot::points2Octree (src/construct.cpp:759) at one rank."""
    if dim != 3:
        raise DendroError(9, "only dim = 3 is implemented")
    ctx = ctx or default_context()
    a, n, on_dev = _points_arg(pts)
    g = np.asarray(gLens, np.float64)
    h = ctypes.c_void_p()
    check(
        ctx.handle,
        ctx._L.dg_points_to_octree(ctx.handle, _ptr(a), n, _ptr(g), maxDepth, maxNumPtsPerOctant, comm_size, on_dev,
                                   ctypes.byref(h)),
        "points2Octree",
    )
    return Octree(ctx, h)


def points2OctreeBatch(clouds, gLens=(1.0, 1.0, 1.0), maxDepth: int = 30, maxNumPtsPerOctant: int = 1,
                       ctx: Context | None = None, seg_start=None) -> Octree:
    """points2Octree over a batch of clouds in one pass.

    ``clouds`` is a list of (n_s, 3) arrays, or one concatenated array / CUDA
    tensor together with ``seg_start`` (nseg + 1 offsets).
    """
    ctx = ctx or default_context()
    if seg_start is None:
        sizes = [len(c) for c in clouds]
        seg_start = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
        pts = np.concatenate([np.asarray(c, np.float64).reshape(-1, 3) for c in clouds]) if sizes else np.zeros((0, 3))
    else:
        pts = clouds
        seg_start = np.ascontiguousarray(seg_start, dtype=np.uint64)
    a, n, on_dev = _points_arg(pts)
    g = np.asarray(gLens, np.float64)
    h = ctypes.c_void_p()
    check(ctx.handle,
          ctx._L.dg_points_to_octree_batch(ctx.handle, _ptr(a), n, _ptr(seg_start), len(seg_start) - 1, _ptr(g), maxDepth,
                                           maxNumPtsPerOctant, on_dev, ctypes.byref(h)),
          "points2OctreeBatch")
    return Octree(ctx, h)


def sortUniquePoints(pts, gLens=(1.0, 1.0, 1.0), maxDepth: int = 30, ctx: Context | None = None) -> np.ndarray:
    """par::removeDuplicates over the level-maxDepth point octants (Morton sort + unique)."""
    ctx = ctx or default_context()
    a, n, on_dev = _points_arg(pts)
    g = np.asarray(gLens, np.float64)
    out = np.empty((max(n, 1), 4), np.uint32)
    nu = ctypes.c_size_t()
    check(ctx.handle, ctx._L.dg_sort_unique_points(ctx.handle, _ptr(a), n, _ptr(g), maxDepth, on_dev, _ptr(out), 0, ctypes.byref(nu)),
          "sortUniquePoints")
    return out[: nu.value].copy()


def balanceOctree(octree: Octree, dim: int = 3, maxDepth: int | None = None, incCorner: bool = True,
                  comm_size: int = 1) -> Octree:
    """ot::balanceOctree (src/balance.cpp:31) at one rank; the input is kept."""
    if dim != 3:
        raise DendroError(9, "only dim = 3 is implemented")
    if maxDepth is not None and maxDepth != octree.max_depth:
        raise DendroError(1, "maxDepth differs from the octree's")
    ctx = octree.ctx
    h = ctypes.c_void_p()
    check(ctx.handle, ctx._L.dg_balance_octree(ctx.handle, octree.handle, 1 if incCorner else 0, comm_size, ctypes.byref(h)),
          "balanceOctree")
    return Octree(ctx, h)


def coarsenOctree(octree: Octree) -> Octree:
    """ot::coarsenOctree (src/coarsen.cpp:53): merge every complete family of 8 leaves."""
    ctx = octree.ctx
    h = ctypes.c_void_p()
    check(ctx.handle, ctx._L.dg_coarsen_octree(ctx.handle, octree.handle, ctypes.byref(h)), "coarsenOctree")
    return Octree(ctx, h)


class DA:
    """ot::DA (src/oda/oda.cpp:250) at one rank, device resident."""

    def __init__(self, octree: Octree):
        ctx = octree.ctx
        self.ctx = ctx
        self.max_depth = octree.max_depth
        h = ctypes.c_void_p()
        check(ctx.handle, ctx._L.dg_da_build(ctx.handle, octree.handle, ctypes.byref(h)), "DA")
        self.handle = h
        ne, nn = ctypes.c_size_t(), ctypes.c_size_t()
        ctx._L.dg_da_sizes(h, ctypes.byref(ne), ctypes.byref(nn))
        self.n_elem, self.n_node = ne.value, nn.value

    def getElementSize(self) -> int:
        return self.n_elem

    def getNodeSize(self) -> int:
        return self.n_node

    def download(self) -> dict:
        meta = np.empty(max(self.n_elem, 1), np.uint32)
        nodes = np.empty((max(self.n_elem, 1), 8), np.uint32)
        xyz = np.empty((max(self.n_node, 1), 3), np.uint32)
        check(self.ctx.handle, self.ctx._L.dg_da_download(self.ctx.handle, self.handle, _ptr(meta), _ptr(nodes), _ptr(xyz), 0),
              "dg_da_download")
        meta = meta[: self.n_elem]
        return {
            "level": (meta & 255).astype(np.uint8),
            "child": ((meta >> 8) & 255).astype(np.uint8),
            "hmask": ((meta >> 16) & 255).astype(np.uint8),
            "etype": (meta >> 24).astype(np.uint8),
            "nodes": nodes[: self.n_elem],
            "node_xyz": xyz[: self.n_node],
        }

    def matvec(self, x, out=None, precision: int = 64, lapFac: float = 1.0, massFac: float = 1.0):
        """Jacobian1MatMult (examples/src/backend/odaJac.C:294): out = (lapFac*L + massFac*M) x."""
        on_dev = 1 if _is_device(x) else 0
        if on_dev:
            if out is None:
                out = x.new_empty(x.shape)
        else:
            x = np.ascontiguousarray(x, dtype=np.float64 if precision == 64 else np.float32)
            if out is None:
                out = np.empty_like(x)
        if (x.numel() if on_dev else x.size) != self.n_node:
            raise ValueError("vector length differs from the node count")
        check(self.ctx.handle,
              self.ctx._L.dg_matvec(self.ctx.handle, self.handle, _ptr(x), _ptr(out), precision, lapFac, massFac, on_dev),
              "Jacobian1MatMult")
        return out

    def free(self):
        if getattr(self, "handle", None):
            self.ctx._L.dg_da_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
