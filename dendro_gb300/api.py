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
    "MultiGrid",
    "default_context",
    "readPtsFromFile",
    "writePtsToFile",
    "readNodesFromFile",
    "writeNodesToFile",
    "readNodesFromFile_binary",
    "writeNodesToFile_binary",
]


def _is_device(a) -> bool:
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _check_len(x, n: int, what: str) -> None:
    """Host and device vectors must hold exactly n entries: the C ABI takes
    plain pointers and cannot check their lengths."""
    m = x.numel() if _is_device(x) else np.asarray(x).size
    if m != n:
        raise ValueError(f"{what}: vector of {m} entries where the mesh has {n} nodes")


def _ptr(a):
    """Address of an argument.  A CUDA tensor may still be being written by
    torch on torch's current stream, while the library works on its own
    stream: wait for torch's stream first, so the library reads finished data
    (every library call itself returns with its results complete)."""
    if _is_device(a):
        import torch

        torch.cuda.current_stream(a.device).synchronize()
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

    def set_matvec_form(self, form: str):
        """FP32 element loop form: "runs" (default) or "pairs"."""
        check(self.handle, self._L.dg_ctx_set_matvec_form(self.handle, {"runs": 0, "pairs": 1}[form]),
              "set_matvec_form")

    def set_order(self, order: str):
        """Order of octant records at the boundary: "morton" (default) or
        "hilbert" (the reference's default HILBERT_ORDERING build)."""
        code = {"morton": 0, "hilbert": 1}[order]
        check(self.handle, self._L.dg_ctx_set_order(self.handle, code), "dg_ctx_set_order")

    @property
    def order(self) -> str:
        v = ctypes.c_int()
        check(self.handle, self._L.dg_ctx_get_order(self.handle, ctypes.byref(v)), "dg_ctx_get_order")
        return ("morton", "hilbert")[v.value]

    def autotune_log(self) -> str:
        """The autotuner's decisions on this context, one line each."""
        return self._L.dg_ctx_autotune_log(self.handle).decode()

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

    def extract(self, seg: int) -> "Octree":
        """Cloud ``seg`` of a batch as its own device-resident octree."""
        h = ctypes.c_void_p()
        check(self.ctx.handle, self.ctx._L.dg_octree_extract(self.ctx.handle, self.handle, seg, ctypes.byref(h)), "extract")
        return Octree(self.ctx, h)

    def split(self) -> list:
        """The octree of every cloud, as (n_s, 4) uint32 arrays."""
        a = self.to_numpy()
        off = self.segments()
        return [a[off[i]:off[i + 1]] for i in range(len(off) - 1)]

    def to_numpy(self, ctx: "Context | None" = None) -> np.ndarray:
        """The records on the host, downloaded through ``ctx`` (default: the
        context that made the octree; a context serves one host thread at a
        time, so a worker thread passes its own)."""
        c = ctx or self.ctx
        out = np.empty((self.size, 4), np.uint32)
        check(c.handle, c._L.dg_octree_download(c.handle, self.handle, _ptr(out), 0), "dg_octree_download")
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

    def free(self, ctx: "Context | None" = None):
        """Release the device memory (on ``ctx``'s stream when given)."""
        if self.handle:
            c = ctx or self.ctx
            c._L.dg_octree_free(c.handle, self.handle)
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
        if sizes and all(_is_device(c) for c in clouds):
            import torch

            pts = torch.cat([c.reshape(-1, 3) for c in clouds]).contiguous()
        else:
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


def _path(p) -> bytes:
    import os

    return os.fsencode(p)


def readPtsFromFile(path, device: bool = False, ctx: Context | None = None):
    """ot::readPtsFromFile (src/octFunctions.cpp:319): the points of a .pts
    file, (n, 3) FP64 -- numpy, or with ``device`` a CUDA tensor filled
    through pinned staging buffers."""
    ctx = ctx or default_context()
    n = ctypes.c_size_t()
    check(None, ctx._L.dg_pts_file_count(_path(path), ctypes.byref(n)), "readPtsFromFile")
    if device:
        import torch

        out = torch.empty((n.value, 3), dtype=torch.float64, device=f"cuda:{ctx.device}")
    else:
        out = np.empty((n.value, 3), np.float64)
    got = ctypes.c_size_t()
    check(ctx.handle, ctx._L.dg_pts_file_read(ctx.handle, _path(path), _ptr(out), n.value, 1 if device else 0,
                                              ctypes.byref(got)), "readPtsFromFile")
    return out[: got.value]


def writePtsToFile(path, pts, ctx: Context | None = None):
    """ot::writePtsToFile (src/octFunctions.cpp:380); pts is (n, 3) FP64,
    numpy or a CUDA tensor."""
    ctx = ctx or default_context()
    a, n, on_dev = _points_arg(pts)
    check(ctx.handle, ctx._L.dg_pts_file_write(ctx.handle, _path(path), _ptr(a), n, on_dev), "writePtsToFile")


def writeNodesToFile(path, octree: Octree):
    """ot::writeNodesToFile (src/octFunctions.cpp:496): text, byte for byte
    as the reference writes it; the lines are formatted on the GPU."""
    check(octree.ctx.handle, octree.ctx._L.dg_octree_write_text(octree.ctx.handle, octree.handle, _path(path)),
          "writeNodesToFile")


def writeNodesToFile_binary(path, octree: Octree):
    """ot::writeNodesToFile_binary (src/octFunctions.cpp:482): 28-byte records."""
    check(octree.ctx.handle, octree.ctx._L.dg_octree_write_binary(octree.ctx.handle, octree.handle, _path(path)),
          "writeNodesToFile_binary")


def readNodesFromFile(path, ctx: Context | None = None) -> Octree:
    """ot::readNodesFromFile (src/octFunctions.cpp:452): the octants of a text
    file, in the file's order, parsed on the GPU."""
    ctx = ctx or default_context()
    h = ctypes.c_void_p()
    check(ctx.handle, ctx._L.dg_octree_read_text(ctx.handle, _path(path), ctypes.byref(h)), "readNodesFromFile")
    return Octree(ctx, h)


def readNodesFromFile_binary(path, ctx: Context | None = None) -> Octree:
    """ot::readNodesFromFile_binary (src/octFunctions.cpp:435): the file's
    records (the reference's reader repeats the last one)."""
    ctx = ctx or default_context()
    h = ctypes.c_void_p()
    check(ctx.handle, ctx._L.dg_octree_read_binary(ctx.handle, _path(path), ctypes.byref(h)),
          "readNodesFromFile_binary")
    return Octree(ctx, h)


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


def sortOctants(octants, maxDepth: int = 30, removeDuplicates: bool = False, ctx: Context | None = None) -> np.ndarray:
    """par::sampleSort / par::removeDuplicates (include/parUtils.h:424,437)
    of n x 4 uint32 octant records, in the context's octant order."""
    ctx = ctx or default_context()
    a = np.ascontiguousarray(octants, dtype=np.uint32).reshape(-1, 4)
    out = np.empty((max(a.shape[0], 1), 4), np.uint32)
    n = ctypes.c_size_t()
    check(ctx.handle, ctx._L.dg_sort_octants(ctx.handle, _ptr(a), a.shape[0], maxDepth, int(removeDuplicates), 0,
                                             _ptr(out), 0, ctypes.byref(n)), "sortOctants")
    return out[: n.value]


TS_SORT_ONLY, TS_REMOVE_DUPLICATES, TS_CONSTRUCT_OCTREE, TS_BALANCE_OCTREE = 0, 1, 2, 4


def treeSort(octants, maxDepth: int = 30, options: int = TS_REMOVE_DUPLICATES, ctx: Context | None = None) -> np.ndarray:
    """SFC::parSort::SFC_treeSort (include/sfcSort.h:1378) at one rank on
    n x 4 uint32 octant records: TS_SORT_ONLY sorts them (the reference's
    pNodes, sorted in place); TS_REMOVE_DUPLICATES also removes repeated
    octants and every octant with a descendant in the input (pOutSorted,
    sfcSort.h:532-575).  Records come back in the context's octant order."""
    ctx = ctx or default_context()
    a = np.ascontiguousarray(octants, dtype=np.uint32).reshape(-1, 4)
    out = np.empty((max(a.shape[0], 1), 4), np.uint32)
    n = ctypes.c_size_t()
    check(ctx.handle, ctx._L.dg_tree_sort(ctx.handle, _ptr(a), a.shape[0], maxDepth, int(options), 0, _ptr(out), 0,
                                          ctypes.byref(n)), "SFC_treeSort")
    return out[: n.value]


def completeOctree(octants, maxDepth: int = 30, isUnique: bool = False, isSorted: bool = False,
                   ctx: Context | None = None) -> Octree:
    """ot::completeOctree (src/construct.cpp:518) at one rank.  ``octants``:
    n x 4 uint32 records {x, y, z, level} (numpy array or CUDA tensor).  Not
    declared unique: sorted, duplicates and octants with a descendant in the
    input dropped; gaps filled with the coarsest octants."""
    ctx = ctx or default_context()
    dev = _is_device(octants)
    a = octants if dev else np.ascontiguousarray(octants, dtype=np.uint32).reshape(-1, 4)
    n = a.shape[0] if a.ndim > 1 else a.shape[0] // 4
    h = ctypes.c_void_p()
    check(ctx.handle, ctx._L.dg_complete_octree(ctx.handle, _ptr(a), n, maxDepth, int(isUnique), int(isSorted),
                                                1 if dev else 0, ctypes.byref(h)), "completeOctree")
    return Octree(ctx, h)


class Csr:
    """An assembled operator on the device (dg_csr): CSR over the DA's node
    ids, columns sorted within each row, FP64 values."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx, self.handle = ctx, handle
        n, z, mr = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_uint()
        check(ctx.handle, ctx._L.dg_csr_sizes(handle, ctypes.byref(n), ctypes.byref(z), ctypes.byref(mr)),
              "dg_csr_sizes")
        self.n_rows, self.nnz, self.max_row_len = n.value, z.value, mr.value

    def to_numpy(self):
        """(row_ptr int64[n_rows + 1], col uint32[nnz], val float64[nnz])"""
        rp = np.empty(self.n_rows + 1, np.int64)
        col = np.empty(max(self.nnz, 1), np.uint32)
        val = np.empty(max(self.nnz, 1), np.float64)
        check(self.ctx.handle, self.ctx._L.dg_csr_download(self.ctx.handle, self.handle, _ptr(rp), _ptr(col), _ptr(val), 0),
              "dg_csr_download")
        return rp, col[: self.nnz], val[: self.nnz]

    def to_scipy(self):
        import scipy.sparse as sp

        rp, col, val = self.to_numpy()
        return sp.csr_matrix((val, col.astype(np.int64), rp), shape=(self.n_rows, self.n_rows))

    def spmv(self, x, out=None):
        """y = A x (FP64); host arrays or CUDA tensors."""
        _check_len(x, self.n_rows, "dg_csr_spmv")
        on_dev = _is_device(x)
        if on_dev:
            out = x.new_empty(x.shape) if out is None else out
        else:
            x = np.ascontiguousarray(x, dtype=np.float64)
            out = np.empty_like(x) if out is None else out
        check(self.ctx.handle, self.ctx._L.dg_csr_spmv(self.ctx.handle, self.handle, _ptr(x), _ptr(out), 1 if on_dev else 0),
              "dg_csr_spmv")
        return out

    def free(self):
        if self.handle:
            self.ctx._L.dg_csr_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DA:
    """ot::DA (src/oda/oda.cpp:250) at one rank, device resident."""

    def __init__(self, octree: Octree, compressLut: bool = False):
        ctx = octree.ctx
        self.ctx = ctx
        self.max_depth = octree.max_depth
        self.compressLut = compressLut
        h = ctypes.c_void_p()
        check(ctx.handle, ctx._L.dg_da_build_ex(ctx.handle, octree.handle, int(compressLut), ctypes.byref(h)), "DA")
        self.handle = h
        ne, nn = ctypes.c_size_t(), ctypes.c_size_t()
        ctx._L.dg_da_sizes(h, ctypes.byref(ne), ctypes.byref(nn))
        self.n_elem, self.n_node = ne.value, nn.value

    def getElementSize(self) -> int:
        return self.n_elem

    def assemble(self, lapFac: float = 1.0, massFac: float = 1.0) -> Csr:
        """CreateAndComputeFullJacobian1 (examples/src/backend/odaJac.C:470):
        lapFac K + massFac M as a CSR matrix."""
        h = ctypes.c_void_p()
        check(self.ctx.handle, self.ctx._L.dg_da_assemble(self.ctx.handle, self.handle, lapFac, massFac,
                                                          ctypes.byref(h)), "dg_da_assemble")
        return Csr(self.ctx, h)

    def getNodeSize(self) -> int:
        return self.n_node

    def matvec_coef(self, coef, x, out=None, precision: int = 64):
        """Jacobian2MatMult (examples/src/backend/omgJac.C:1666-1735): per
        element e, coef[e, 0] scales its Laplacian and coef[e, 1] its mass
        (coef: n_elem x 2 FP64, elements in octree order)."""
        on_dev = _is_device(x)
        if on_dev:
            out = x.new_empty(x.shape) if out is None else out
            c = coef
            if c.numel() != 2 * self.n_elem:
                raise ValueError("coef must hold 2 values per element")
        else:
            x = np.ascontiguousarray(x, dtype=np.float64 if precision == 64 else np.float32)
            out = np.empty_like(x) if out is None else out
            c = self._coef(coef)
        _check_len(x, self.n_node, "Jacobian2MatMult")
        check(self.ctx.handle, self.ctx._L.dg_matvec_coef(self.ctx.handle, self.handle, _ptr(c), _ptr(x), _ptr(out),
                                                          precision, 1 if on_dev else 0), "dg_matvec_coef")
        return out

    def _coef(self, coef) -> np.ndarray:
        """Per-element (lap, mass) factors as an n_elem x 2 FP64 host array."""
        c = np.ascontiguousarray(coef, dtype=np.float64).reshape(-1, 2)
        if c.shape[0] != self.n_elem:
            raise ValueError("coef must hold 2 values per element")
        return c

    def diagonal(self, lapFac: float = 1.0, massFac: float = 1.0, coef=None) -> np.ndarray:
        """Jacobian1MatGetDiagonal (odaJac.C:160-222), or with coef
        Jacobian2MatGetDiagonal (omgJac.C:1641); FP64, host array."""
        d = np.empty(max(self.n_node, 1), np.float64)
        c = None if coef is None else self._coef(coef)
        check(self.ctx.handle, self.ctx._L.dg_da_diagonal(self.ctx.handle, self.handle, None if c is None else _ptr(c),
                                                          lapFac, massFac, _ptr(d), 0), "dg_da_diagonal")
        return d[: self.n_node]

    def assemble_coef(self, coef) -> "Csr":
        """BUILD_FULL_JAC_TYPE2_BLOCK (omgJac.C:1804-1858): the per-element
        operator of matvec_coef as a CSR matrix."""
        c = self._coef(coef)
        h = ctypes.c_void_p()
        check(self.ctx.handle, self.ctx._L.dg_da_assemble_coef(self.ctx.handle, self.handle, _ptr(c), 0, ctypes.byref(h)),
              "dg_da_assemble_coef")
        return Csr(self.ctx, h)

    def memory_bytes(self) -> int:
        """Device bytes the DA holds."""
        b = ctypes.c_size_t()
        check(self.ctx.handle, self.ctx._L.dg_da_memory(self.handle, ctypes.byref(b)), "dg_da_memory")
        return b.value

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


class MultiGrid:
    """Geometric multigrid hierarchy and solver (the reference's DAMG, omg module).

    Levels: the given balanced octree, then coarsenOctree + balanceOctree
    until a level holds at most ``max_coarse_elems`` elements
    (src/omg/blockDiag.cpp:1312).  Operator: -lap(u) + u with u = 0 on the
    boundary of the unit cube (DirichletJacobianMatMult,
    examples/src/backend/omgJac.C:958).
    """

    def __init__(self, octree: Octree, max_coarse_elems: int = 4096, ctx: Context | None = None):
        ctx = ctx or octree.ctx
        self.ctx = ctx
        self.max_depth = octree.max_depth
        h = ctypes.c_void_p()
        check(ctx.handle, ctx._L.dg_mg_setup(ctx.handle, octree.handle, max_coarse_elems, ctypes.byref(h)), "MultiGrid")
        self.handle = h
        n = ctypes.c_size_t()
        ctx._L.dg_mg_levels(h, ctypes.byref(n))
        self.n_levels = n.value
        self.sizes = []
        for l in range(self.n_levels):
            e, v = ctypes.c_size_t(), ctypes.c_size_t()
            ctx._L.dg_mg_level_sizes(h, l, ctypes.byref(e), ctypes.byref(v))
            self.sizes.append((e.value, v.value))

    def diagonal(self, level: int) -> np.ndarray:
        """DirichletJacobianMatGetDiagonal (omgJac.C:1111): FP64, 1 on boundary nodes."""
        n = self.sizes[level][1]
        d = np.empty(max(n, 1), np.float64)
        check(self.ctx.handle, self.ctx._L.dg_mg_diagonal(self.ctx.handle, self.handle, level, _ptr(d), 0),
              "dg_mg_diagonal")
        return d[:n]

    def assemble(self, level: int) -> Csr:
        """ComputeDirichletJacobian (examples/src/backend/omgJac.C:383): the
        Dirichlet operator of a level as a CSR matrix."""
        h = ctypes.c_void_p()
        check(self.ctx.handle, self.ctx._L.dg_mg_assemble(self.ctx.handle, self.handle, level, ctypes.byref(h)),
              "dg_mg_assemble")
        return Csr(self.ctx, h)

    def level_nodes(self, level: int, device: bool = False):
        """Node coordinates (n_node, 3) of a level: numpy uint32, or with
        ``device`` an int32 CUDA tensor holding the same bits."""
        if device:
            import torch

            xyz = torch.empty((self.sizes[level][1], 3), dtype=torch.int32, device=f"cuda:{self.ctx.device}")
        else:
            xyz = np.empty((self.sizes[level][1], 3), np.uint32)
        check(self.ctx.handle,
              self.ctx._L.dg_mg_level_nodes(self.ctx.handle, self.handle, level, _ptr(xyz), 1 if device else 0),
              "level_nodes")
        return xyz

    def level_octree(self, level: int) -> np.ndarray:
        out = np.empty((self.sizes[level][0], 4), np.uint32)
        check(self.ctx.handle, self.ctx._L.dg_mg_level_octree(self.ctx.handle, self.handle, level, _ptr(out), 0), "level_octree")
        return out

    def _op(self, fn, level, x, n_in, n_out, precision):
        _check_len(x, n_in, fn.__name__)
        on_dev = 1 if _is_device(x) else 0
        if on_dev:
            out = x.new_empty((n_out,))
        else:
            x = np.ascontiguousarray(x, dtype=np.float32 if precision == 32 else np.float64)
            out = np.empty(n_out, x.dtype)
        check(self.ctx.handle, fn(self.ctx.handle, self.handle, level, _ptr(x), _ptr(out), precision, on_dev), fn.__name__)
        return out

    def matvec(self, level: int, x, precision: int = 64):
        """DirichletJacobianMatMult on a level: FP64 (64), FP32 (32), or FP64
        vectors in double-single arithmetic (48)."""
        n = self.sizes[level][1]
        return self._op(self.ctx._L.dg_mg_matvec, level, x, n, n, precision)

    def restrict(self, fine_level: int, x, precision: int = 64):
        """restrictMatVecType1: fine level -> next coarser level."""
        return self._op(self.ctx._L.dg_mg_restrict, fine_level, x, self.sizes[fine_level][1],
                        self.sizes[fine_level + 1][1], precision)

    def prolong(self, fine_level: int, x, precision: int = 64):
        """prolongMatVecType1: next coarser level -> fine level."""
        return self._op(self.ctx._L.dg_mg_prolong, fine_level, x, self.sizes[fine_level + 1][1],
                        self.sizes[fine_level][1], precision)

    def set_smoother(self, omega: float = 0.667, nu_pre: int = 2, nu_post: int = 2):
        check(self.ctx.handle, self.ctx._L.dg_mg_set_smoother(self.handle, omega, nu_pre, nu_post), "set_smoother")

    def set_cg_operator(self, precision: int = 48, reliable_delta: float = 1e-3):
        """The CG's operator q = A p with an FP32 V-cycle: double-single
        arithmetic on FP64 vectors (48, the default), FP64 (64), or FP32
        with FP64 residual replacement (32)."""
        check(self.ctx.handle, self.ctx._L.dg_mg_set_cg_operator(self.handle, precision, reliable_delta),
              "set_cg_operator")

    def rhs(self, f):
        """Load vector b = M f of a nodal field on the finest level, 0 on the boundary."""
        _check_len(f, self.sizes[0][1], "rhs")
        on_dev = 1 if _is_device(f) else 0
        if on_dev:
            out = f.new_empty(f.shape)
        else:
            f = np.ascontiguousarray(f, dtype=np.float64)
            out = np.empty_like(f)
        check(self.ctx.handle, self.ctx._L.dg_mg_rhs(self.ctx.handle, self.handle, _ptr(f), _ptr(out), on_dev), "rhs")
        return out

    def solve(self, b, precision: int = 32, rtol: float = 1e-8, maxit: int = 200, x=None):
        """CG preconditioned by one V-cycle (FP32 or FP64) per iteration; FP64 residuals.

        Returns (x, iterations, final FP64 relative residual).
        """
        _check_len(b, self.sizes[0][1], "solve")
        if x is not None:
            _check_len(x, self.sizes[0][1], "solve (x)")
        on_dev = 1 if _is_device(b) else 0
        if on_dev:
            x = b.new_empty(b.shape) if x is None else x
        else:
            b = np.ascontiguousarray(b, dtype=np.float64)
            x = np.empty_like(b) if x is None else x
        it, rr = ctypes.c_int(), ctypes.c_double()
        check(self.ctx.handle,
              self.ctx._L.dg_mg_solve(self.ctx.handle, self.handle, _ptr(b), _ptr(x), precision, rtol, maxit, on_dev,
                                      ctypes.byref(it), ctypes.byref(rr)), "solve")
        return x, it.value, rr.value

    def free(self):
        if getattr(self, "handle", None):
            self.ctx._L.dg_mg_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
