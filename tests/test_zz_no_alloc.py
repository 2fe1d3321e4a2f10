"""dg_sort_unique_points_noalloc (static device scratch, no allocation in the
call) against dg_sort_unique_points through the C ABI: the unique sorted
point octants must be identical (integer records: exact), on two calls in
a row, for every case.  The file is collected last so that it also runs
after everything else has used the device."""
import ctypes

import numpy as np
import pytest

from dendro_gb300 import _lib, datagen

DG_OK, DG_ERR_INVALID_ARG, DG_ERR_DOMAIN, DG_ERR_CAPACITY = 0, 1, 4, 10
NMAX = 1 << 20


def _L():
    return _lib.load()


def _noalloc(L, xyz_ptr, n, g, D, out_ptr, stream=None):
    nu = ctypes.c_size_t(12345)
    rc = L.dg_sort_unique_points_noalloc(xyz_ptr, n, g.ctypes.data, D, out_ptr, ctypes.byref(nu), stream)
    return rc, nu.value


def test_capacity_and_empty_rejected_before_any_device_work():
    """Both paths return before touching CUDA, so they run without a GPU."""
    L = _L()
    assert "#define DG_NOALLOC_MAX_POINTS ((size_t)1 << 20)" in open(_lib.HEADER).read()
    g = np.ones(3)
    rc, _ = _noalloc(L, 16, NMAX + 1, g, 30, 16)
    assert rc == DG_ERR_CAPACITY
    assert "capacity" in L.dg_status_string(rc).decode()
    rc, nu = _noalloc(L, None, 0, g, 30, None)
    assert rc == DG_OK and nu == 0
    rc, _ = _noalloc(L, 16, 5, g, 31, 16)  # maxDepth > 30
    assert rc == DG_ERR_INVALID_ARG


def _cases():
    rng = np.random.Generator(np.random.PCG64(11))
    dup = np.repeat(datagen.lognormal(50_000, seed=5), 8, axis=0)
    rng.shuffle(dup)
    return [
        ("lognormal300k_D30", datagen.lognormal(300_000, seed=1), 30),
        ("mixture_dups_D8", datagen.mixture(400_000, rng), 8),
        ("repeated_D30", dup, 30),
        ("max_size_D20", datagen.lognormal(NMAX, seed=2), 20),
        ("single_D30", datagen.lognormal(1, seed=3), 30),
        ("tiny_D0", datagen.lognormal(1000, seed=4), 0),
    ]


@pytest.mark.gpu
@pytest.mark.parametrize("name,pts,D", _cases(), ids=[c[0] for c in _cases()])
def test_noalloc_equals_allocating_entry(name, pts, D):
    torch = pytest.importorskip("torch")
    L = _L()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(0)
    n = len(pts)
    g = np.ones(3)
    xyz = torch.from_numpy(np.ascontiguousarray(pts, np.float64)).to(dev)
    ref = torch.zeros((n, 4), dtype=torch.int32, device=dev)
    ctx = ctypes.c_void_p()
    assert L.dg_ctx_create(0, ctypes.byref(ctx)) == DG_OK
    try:
        nref = ctypes.c_size_t()
        torch.cuda.synchronize()
        rc = L.dg_sort_unique_points(ctx, xyz.data_ptr(), n, g.ctypes.data, D, 1, ref.data_ptr(), 1,
                                     ctypes.byref(nref))
        assert rc == DG_OK, L.dg_ctx_last_error(ctx)
    finally:
        L.dg_ctx_destroy(ctx)
    want = ref[: nref.value].cpu().numpy()
    for call in range(2):  # two calls in a row reuse the same scratch
        out = torch.full((n, 4), -1 - call, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        rc, nu = _noalloc(L, xyz.data_ptr(), n, g, D, out.data_ptr())
        assert rc == DG_OK, L.dg_status_string(rc)
        assert nu == nref.value
        np.testing.assert_array_equal(out[:nu].cpu().numpy(), want)
        # nothing written past the unique records
        assert bool((out[nu:] == -1 - call).all())


@pytest.mark.gpu
def test_noalloc_errors_leave_the_scratch_usable():
    torch = pytest.importorskip("torch")
    L = _L()
    dev = torch.device("cuda:0")
    g = np.ones(3)
    pts = datagen.lognormal(5000, seed=9)
    bad = pts.copy()
    bad[1234] = (0.5, 1.5, 0.5)  # outside the unit cube
    xb = torch.from_numpy(bad).to(dev)
    out = torch.zeros((5000, 4), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc, _ = _noalloc(L, xb.data_ptr(), 5000, g, 30, out.data_ptr())
    assert rc == DG_ERR_DOMAIN
    # a misaligned output pointer is refused before any work
    rc, _ = _noalloc(L, xb.data_ptr(), 5000, g, 30, out.data_ptr() + 4)
    assert rc == DG_ERR_INVALID_ARG
    # the next valid call succeeds and matches the allocating entry point
    xg = torch.from_numpy(pts).to(dev)
    torch.cuda.synchronize()
    rc, nu = _noalloc(L, xg.data_ptr(), 5000, g, 30, out.data_ptr())
    assert rc == DG_OK
    ctx = ctypes.c_void_p()
    assert L.dg_ctx_create(0, ctypes.byref(ctx)) == DG_OK
    try:
        ref = np.zeros((5000, 4), np.uint32)
        nref = ctypes.c_size_t()
        assert L.dg_sort_unique_points(ctx, pts.ctypes.data, 5000, g.ctypes.data, 30, 0, ref.ctypes.data, 0,
                                       ctypes.byref(nref)) == DG_OK
    finally:
        L.dg_ctx_destroy(ctx)
    assert nu == nref.value
    np.testing.assert_array_equal(out[:nu].cpu().numpy().view(np.uint32), ref[:nu])


def test_noalloc_source_allocates_nothing():
    """No allocating call appears in the entry point's translation unit (a
    pooled buffer, cudaMalloc / cudaMallocAsync / cudaFree or a library
    routine that allocates)."""
    import os
    import re

    src = open(os.path.join(os.path.dirname(_lib.HEADER), "..", "dendro_gb300", "csrc", "dg_noalloc.cu")).read()
    code = re.sub(r"//[^\n]*", "", src)
    for pat in (r"\bcudaMalloc", r"\bcudaFree", r"\bDBuf\b", r"\bcudaMallocManaged", r"\bcudaHostAlloc", r"\bnew\b",
                r"\bmalloc\(", r"\bthrust::", r"\bcub::"):
        assert not re.search(pat, code), pat


@pytest.mark.gpu
def test_noalloc_device_memory_unchanged_by_a_call():
    """After a warm-up call, a further call leaves the device's free memory
    exactly as it was (cudaMemGetInfo before and after)."""
    torch = pytest.importorskip("torch")
    L = _L()
    dev = torch.device("cuda:0")
    g = np.ones(3)
    pts = datagen.lognormal(200_000, seed=12)
    xyz = torch.from_numpy(pts).to(dev)
    out = torch.zeros((len(pts), 4), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc, nu = _noalloc(L, xyz.data_ptr(), len(pts), g, 30, out.data_ptr())
    assert rc == DG_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    rc, nu2 = _noalloc(L, xyz.data_ptr(), len(pts), g, 30, out.data_ptr())
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert rc == DG_OK and nu2 == nu
    assert free1 == free0
