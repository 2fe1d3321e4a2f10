"""The C ABI library builds, loads and exports every declared symbol (CPU only;
no compute call is made without a GPU)."""
import ctypes
import os
import subprocess

import pytest

from dendro_gb300 import _lib
from dendro_gb300 import build as cuda_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_builds_for_sm103a():
    path = cuda_build.build()
    assert os.path.exists(path)
    assert "arch=compute_103a,code=sm_103a" in " ".join(cuda_build.NVCC_FLAGS)


def test_exports_every_header_symbol():
    L = _lib.load()
    names = _lib.header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_exported_symbols_are_c_linkage():
    out = subprocess.run(["nm", "-D", "--defined-only", cuda_build.LIB], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for n in _lib.header_functions():
        assert n in exported, n


def test_status_strings_without_gpu():
    L = _lib.load()
    assert L.dg_version() >= 1
    assert L.dg_status_string(0) == b"ok"
    assert L.dg_status_string(8) == b"communicator size must be 1"


def test_invalid_arguments_rejected_before_any_gpu_work():
    L = _lib.load()
    # null context / null outputs return DG_ERR_INVALID_ARG without touching a device
    assert L.dg_ctx_destroy(None) == 1
    out = ctypes.c_void_p()
    assert L.dg_points_to_octree(None, None, 0, None, 30, 1, 1, 0, ctypes.byref(out)) == 1
    assert L.dg_points_to_octree(None, None, 0, (ctypes.c_double * 3)(1, 1, 1), 30, 1, 2, 0, ctypes.byref(out)) == 8
    assert L.dg_matvec(None, None, None, None, 64, 1.0, 1.0, 0) == 1
    # the entry points beside the hot path check their arguments the same way
    rec = (ctypes.c_uint32 * 4)(0, 0, 0, 0)
    n = ctypes.c_size_t()
    assert L.dg_complete_octree(None, rec, 1, 30, 0, 0, 0, None) == 1          # no output handle
    assert L.dg_complete_octree(None, rec, 1, 31, 0, 0, 0, ctypes.byref(out)) == 1  # maxDepth > 30
    assert L.dg_sort_octants(None, rec, 1, 30, 0, 0, None, 0, ctypes.byref(n)) == 1
    assert L.dg_da_assemble(None, None, 1.0, 1.0, ctypes.byref(out)) == 1
    assert L.dg_mg_assemble(None, None, 0, ctypes.byref(out)) == 1
    assert L.dg_csr_sizes(None, None, None, None) == 1
    assert L.dg_csr_free(None, None) == 0
    assert L.dg_matvec_coef(None, None, None, None, None, 64, 0) == 1
    assert L.dg_da_diagonal(None, None, None, 1.0, 1.0, None, 0) == 1
    assert L.dg_mg_diagonal(None, None, 0, None, 0) == 1
    assert L.dg_da_memory(None, None) == 1
    assert L.dg_ctx_set_order(None, 1) == 1
    assert L.dg_da_build_ex(None, None, 1, ctypes.byref(out)) == 1


def test_product_fails_loudly_without_gpu():
    import dendro_gb300

    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(dendro_gb300.DendroError):
        dendro_gb300.Context(0)


def test_no_oracle_in_product_sources():
    pkg = os.path.join(ROOT, "dendro_gb300")
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in text.replace("the oracle", ""), f


def test_header_is_c99_and_a_c_caller_links(tmp_path):
    """include/dendro_gb300.h compiles as plain C99; a C program links the
    library and calls its context-free entry points (no GPU needed)."""
    import shutil
    import subprocess

    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    lib = _lib.load()._name
    exe = tmp_path / "abi_smoke"
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "c", "abi_smoke.c"), "-o", str(exe), lib,
                           "-Wl,-rpath," + os.path.dirname(lib)])
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    assert '"version"' in r.stdout


def test_cpp_mirror_compiles_cleanly():
    """include/dendro_gb300.hpp with a C++ caller (tests/cpp/dropin_main.cpp):
    no warnings at -Wall -Wextra (compile only; the GPU test runs it)."""
    import shutil
    import subprocess

    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    subprocess.check_call(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                           os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp")])



def test_python_mirror_checks_vector_lengths():
    """The C ABI takes plain pointers, so the Python mirror checks every
    vector's length before a call: a wrong length raises ValueError and
    reaches no native code (the objects here hold sizes only)."""
    from types import SimpleNamespace

    import numpy as np

    from dendro_gb300.api import DA, MultiGrid

    def refuse(*a):
        raise AssertionError("native code reached")

    L = SimpleNamespace(dg_mg_matvec=refuse, dg_mg_restrict=refuse, dg_mg_prolong=refuse, dg_mg_rhs=refuse,
                        dg_mg_solve=refuse, dg_matvec_coef=refuse)
    mg = MultiGrid.__new__(MultiGrid)
    mg.ctx, mg.handle, mg.sizes = SimpleNamespace(_L=L, handle=None), None, [(10, 8), (3, 5)]
    for call in (lambda: mg.matvec(0, np.zeros(7)), lambda: mg.matvec(1, np.zeros(8)),
                 lambda: mg.restrict(0, np.zeros(5)), lambda: mg.prolong(0, np.zeros(8)),
                 lambda: mg.rhs(np.zeros(5)), lambda: mg.solve(np.zeros(9)),
                 lambda: mg.solve(np.zeros(8), x=np.zeros(7))):
        with pytest.raises(ValueError):
            call()
    # the right lengths pass the checks and reach the native call
    for call in (lambda: mg.matvec(0, np.zeros(8)), lambda: mg.matvec(1, np.zeros(5)),
                 lambda: mg.restrict(0, np.zeros(8)), lambda: mg.prolong(0, np.zeros(5)),
                 lambda: mg.rhs(np.zeros(8)), lambda: mg.solve(np.zeros(8), x=np.zeros(8))):
        with pytest.raises(AssertionError, match="native code reached"):
            call()
    da = DA.__new__(DA)
    da.ctx, da.handle, da.n_elem, da.n_node = SimpleNamespace(_L=L, handle=None), None, 2, 6
    with pytest.raises(AssertionError, match="native code reached"):
        da.matvec_coef(np.ones((2, 2)), np.zeros(6))
    with pytest.raises(ValueError):
        da.matvec_coef(np.ones((2, 2)), np.zeros(5))
    with pytest.raises(ValueError):
        da.matvec(np.zeros(5))
    for call in (lambda: da.matvec_coef(np.ones((3, 2)), np.zeros(6)), lambda: da.diagonal(coef=np.ones(2)),
                 lambda: da.assemble_coef(np.ones((1, 2)))):
        with pytest.raises(ValueError):
            call()
    from dendro_gb300.api import Csr

    m = Csr.__new__(Csr)
    m.ctx, m.handle, m.n_rows = SimpleNamespace(_L=SimpleNamespace(dg_csr_spmv=refuse), handle=None), None, 4
    with pytest.raises(ValueError):
        m.spmv(np.zeros(3))
    with pytest.raises(AssertionError, match="native code reached"):
        m.spmv(np.zeros(4))
    mg.handle = da.handle = None  # nothing to free
