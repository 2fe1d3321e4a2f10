"""ctypes binding of libdendro_gb300.so (the C ABI of include/dendro_gb300.h).

The CUDA library is the only implementation: if it cannot be built or
loaded, every entry point raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "dendro_gb300.h")

STATUS = {
    0: "DG_OK",
    1: "DG_ERR_INVALID_ARG",
    2: "DG_ERR_OUT_OF_MEMORY",
    3: "DG_ERR_CUDA",
    4: "DG_ERR_DOMAIN",
    5: "DG_ERR_NOT_BALANCED",
    6: "DG_ERR_TIMEOUT",
    7: "DG_ERR_INTERNAL",
    8: "DG_ERR_COMM_SIZE",
    9: "DG_ERR_UNSUPPORTED",
    10: "DG_ERR_CAPACITY",
}


class DendroError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def header_functions() -> list[str]:
    """Names of every function the public header declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(dg_\w+)\s*\(", text, flags=re.M)))


def _declare(L):
    P = ctypes.c_void_p
    SZ = ctypes.c_size_t
    U = ctypes.c_uint
    I = ctypes.c_int
    PP = ctypes.POINTER(ctypes.c_void_p)
    D = ctypes.c_double
    sig = {
        "dg_version": ([], I),
        "dg_status_string": ([I], ctypes.c_char_p),
        "dg_ctx_create": ([I, PP], I),
        "dg_ctx_destroy": ([P], I),
        "dg_ctx_set_stream": ([P, P], I),
        "dg_ctx_last_error": ([P], ctypes.c_char_p),
        "dg_ctx_autotune_log": ([P], ctypes.c_char_p),
        "dg_ctx_last_device_ms": ([P, ctypes.POINTER(D)], I),
        "dg_ctx_profile": ([P, I], I),
        "dg_ctx_profile_count": ([P, ctypes.POINTER(I)], I),
        "dg_ctx_profile_entry": ([P, I, ctypes.c_char_p, SZ, ctypes.POINTER(D), ctypes.POINTER(ctypes.c_ulonglong),
                                  ctypes.POINTER(D)], I),
        "dg_points_to_octree": ([P, P, SZ, P, U, U, I, I, PP], I),
        "dg_points_to_octree_batch": ([P, P, SZ, P, SZ, P, U, U, I, PP], I),
        "dg_octree_segments": ([P, P, ctypes.POINTER(SZ), P], I),
        "dg_octree_extract": ([P, P, SZ, PP], I),
        "dg_sort_unique_points": ([P, P, SZ, P, U, I, P, I, ctypes.POINTER(SZ)], I),
        "dg_sort_unique_points_noalloc": ([P, SZ, P, U, P, ctypes.POINTER(SZ), P], I),
        "dg_balance_octree": ([P, P, I, I, PP], I),
        "dg_coarsen_octree": ([P, P, PP], I),
        "dg_complete_octree": ([P, P, SZ, U, I, I, I, PP], I),
        "dg_sort_octants": ([P, P, SZ, U, I, I, P, I, ctypes.POINTER(SZ)], I),
        "dg_ctx_set_order": ([P, I], I),
        "dg_ctx_get_order": ([P, ctypes.POINTER(I)], I),
        "dg_octree_size": ([P, ctypes.POINTER(SZ), ctypes.POINTER(U)], I),
        "dg_octree_download": ([P, P, P, I], I),
        "dg_octree_upload": ([P, P, SZ, U, I, PP], I),
        "dg_octree_free": ([P, P], I),
        "dg_pts_file_count": ([ctypes.c_char_p, ctypes.POINTER(SZ)], I),
        "dg_pts_file_read": ([P, ctypes.c_char_p, P, SZ, I, ctypes.POINTER(SZ)], I),
        "dg_pts_file_write": ([P, ctypes.c_char_p, P, SZ, I], I),
        "dg_octree_write_text": ([P, P, ctypes.c_char_p], I),
        "dg_octree_read_text": ([P, ctypes.c_char_p, PP], I),
        "dg_octree_write_binary": ([P, P, ctypes.c_char_p], I),
        "dg_octree_read_binary": ([P, ctypes.c_char_p, PP], I),
        "dg_da_build": ([P, P, PP], I),
        "dg_da_sizes": ([P, ctypes.POINTER(SZ), ctypes.POINTER(SZ)], I),
        "dg_da_download": ([P, P, P, P, P, I], I),
        "dg_da_free": ([P, P], I),
        "dg_matvec": ([P, P, P, P, I, D, D, I], I),
        "dg_da_assemble": ([P, P, D, D, PP], I),
        "dg_da_assemble_coef": ([P, P, P, I, PP], I),
        "dg_matvec_coef": ([P, P, P, P, P, I, I], I),
        "dg_da_diagonal": ([P, P, P, D, D, P, I], I),
        "dg_mg_diagonal": ([P, P, SZ, P, I], I),
        "dg_da_build_ex": ([P, P, I, PP], I),
        "dg_da_memory": ([P, ctypes.POINTER(SZ)], I),
        "dg_mg_assemble": ([P, P, SZ, PP], I),
        "dg_csr_sizes": ([P, ctypes.POINTER(SZ), ctypes.POINTER(SZ), ctypes.POINTER(U)], I),
        "dg_csr_download": ([P, P, P, P, P, I], I),
        "dg_csr_spmv": ([P, P, P, P, I], I),
        "dg_csr_free": ([P, P], I),
        "dg_mg_setup": ([P, P, SZ, PP], I),
        "dg_mg_levels": ([P, ctypes.POINTER(SZ)], I),
        "dg_mg_level_sizes": ([P, SZ, ctypes.POINTER(SZ), ctypes.POINTER(SZ)], I),
        "dg_mg_level_nodes": ([P, P, SZ, P, I], I),
        "dg_mg_level_octree": ([P, P, SZ, P, I], I),
        "dg_mg_matvec": ([P, P, SZ, P, P, I, I], I),
        "dg_mg_restrict": ([P, P, SZ, P, P, I, I], I),
        "dg_mg_prolong": ([P, P, SZ, P, P, I, I], I),
        "dg_mg_set_smoother": ([P, D, I, I], I),
        "dg_mg_set_cg_operator": ([P, I, D], I),
        "dg_mg_rhs": ([P, P, P, P, I], I),
        "dg_mg_solve": ([P, P, P, P, I, D, I, I, ctypes.POINTER(I), ctypes.POINTER(D)], I),
        "dg_mg_free": ([P, P], I),
        "dg_debug_lookback_timeout": ([P, SZ, U], I),
        "dg_tree_sort": ([P, P, SZ, U, U, I, P, I, ctypes.POINTER(SZ)], I),
        "dg_ctx_set_matvec_form": ([P, I], I),
        "dg_dense_spd_inverse": ([P, P, SZ], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res


def load(build_if_needed: bool = True):
    """Load (building first if needed) the CUDA library; raises on failure."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if build_if_needed:
                path = _build.build()
            if not os.path.exists(path):
                raise RuntimeError(f"dendro_gb300 CUDA library missing: {path} (run dendro_gb300.build.build())")
            L = ctypes.CDLL(path)
            _declare(L)
            _lib = L
        return _lib


def check(ctx_handle, status: int, what: str):
    if status != 0:
        L = load()
        msg = L.dg_ctx_last_error(ctx_handle).decode() if ctx_handle else ""
        if not msg:
            msg = L.dg_status_string(status).decode()
        raise DendroError(status, f"{what}: {msg}")
