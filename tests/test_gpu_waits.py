"""The device's bounded waits end with an error status, not a hang: the
radix sort's decoupled look-back is made to wait for a tile that is never
processed (dg_debug_lookback_timeout), gives up after its spin limit, and
the call returns DG_ERR_TIMEOUT; the same context then sorts correctly."""
import ctypes
import time

import numpy as np
import pytest

from dendro_gb300 import _lib, datagen

DG_OK, DG_ERR_INVALID_ARG, DG_ERR_TIMEOUT = 0, 1, 6


@pytest.mark.gpu
def test_lookback_wait_times_out_and_context_recovers():
    L = _lib.load()
    ctx = ctypes.c_void_p()
    assert L.dg_ctx_create(0, ctypes.byref(ctx)) == DG_OK
    try:
        # argument checks first (no kernel runs)
        assert L.dg_debug_lookback_timeout(ctx, 4 * 4096, 0) == DG_ERR_INVALID_ARG
        assert L.dg_debug_lookback_timeout(ctx, 4 * 4096, 4) == DG_ERR_INVALID_ARG
        t0 = time.perf_counter()
        rc = L.dg_debug_lookback_timeout(ctx, 4 * 4096, 1)
        waited = time.perf_counter() - t0
        assert rc == DG_ERR_TIMEOUT, L.dg_status_string(rc)
        assert b"timed out" in L.dg_ctx_last_error(ctx)
        assert waited < 30.0
        # the error word was cleared and the context still works
        pts = datagen.lognormal(100_000, seed=3)
        g = np.ones(3)
        out = np.zeros((len(pts), 4), np.uint32)
        nu = ctypes.c_size_t()
        rc = L.dg_sort_unique_points(ctx, pts.ctypes.data, len(pts), g.ctypes.data, 30, 0, out.ctypes.data, 0,
                                     ctypes.byref(nu))
        assert rc == DG_OK, L.dg_ctx_last_error(ctx)
        from oracle import dg_oracle

        srt = dg_oracle.quantize_sort(pts, 30)
        keep = np.ones(len(srt), bool)
        keep[1:] = np.any(srt[1:] != srt[:-1], axis=1)
        np.testing.assert_array_equal(out[: nu.value], srt[keep])
    finally:
        L.dg_ctx_destroy(ctx)
