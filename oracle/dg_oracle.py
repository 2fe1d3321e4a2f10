"""ctypes front end of the CPU oracle (oracle/dg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of bench.py as the checker.  The shipped library never
imports this module.

Octant arrays are numpy ``uint32`` arrays of shape (n, 4): x, y, z, level.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libdg_oracle.so")
_SRC = os.path.join(_HERE, "dg_oracle.c")


def build(force: bool = False) -> str:
    """Compile the oracle restatement with gcc (seconds)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC):
        os.makedirs(_BUILD, exist_ok=True)
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-o", tmp, _SRC])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class _DA(ctypes.Structure):
    _fields_ = [
        ("n_elem", ctypes.c_size_t),
        ("n_node", ctypes.c_size_t),
        ("child", ctypes.POINTER(ctypes.c_uint8)),
        ("hmask", ctypes.POINTER(ctypes.c_uint8)),
        ("etype", ctypes.POINTER(ctypes.c_uint8)),
        ("level", ctypes.POINTER(ctypes.c_uint8)),
        ("nodes", ctypes.POINTER(ctypes.c_uint32)),
        ("node_xyz", ctypes.POINTER(ctypes.c_uint32)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        P = ctypes.c_void_p
        SZ = ctypes.c_size_t
        U = ctypes.c_uint
        L.dgo_free.argtypes = [P]
        L.dgo_quantize_sort.argtypes = [P, SZ, P, U, ctypes.POINTER(P)]
        L.dgo_points_to_octree.argtypes = [P, SZ, P, U, U, ctypes.POINTER(P), ctypes.POINTER(SZ)]
        L.dgo_p2o_local.argtypes = [P, SZ, U, U, ctypes.POINTER(P), ctypes.POINTER(SZ)]
        L.dgo_balance.argtypes = [P, SZ, U, ctypes.POINTER(P), ctypes.POINTER(SZ)]
        L.dgo_balance_ex.argtypes = [P, SZ, U, ctypes.c_int, ctypes.POINTER(P), ctypes.POINTER(SZ)]
        L.dgo_is_balanced_ex.argtypes = [P, SZ, U, ctypes.c_int]
        L.dgo_coarsen.argtypes = [P, SZ, U, ctypes.POINTER(P), ctypes.POINTER(SZ)]
        L.dgo_hilbert_sort.argtypes = [P, SZ, U]
        L.dgo_complete.argtypes = [P, SZ, U, ctypes.c_int, ctypes.c_int, ctypes.POINTER(P), ctypes.POINTER(SZ)]
        for f in ("dgo_is_sorted_unique", "dgo_is_linear", "dgo_is_complete", "dgo_is_balanced"):
            getattr(L, f).argtypes = [P, SZ, U]
        L.dgo_etype_masks.argtypes = [P]
        L.dgo_stencils.argtypes = [P, P]
        L.dgo_da_build.argtypes = [P, SZ, U, ctypes.POINTER(_DA)]
        L.dgo_da_free.argtypes = [ctypes.POINTER(_DA)]
        L.dgo_matvec.argtypes = [ctypes.POINTER(_DA), U, P, P, ctypes.c_double, ctypes.c_double]
        L.dgo_dirichlet_matvec.argtypes = [ctypes.POINTER(_DA), U, P, P]
        L.dgo_dirichlet_diag.argtypes = [ctypes.POINTER(_DA), U, P]
        L.dgo_prolong_map.argtypes = [ctypes.POINTER(_DA), P, SZ, ctypes.POINTER(_DA), U, P, P]
        L.dgo_rmat_tables.argtypes = [P, P]
        L.dgo_fnv1a.argtypes = [P, SZ]
        L.dgo_fnv1a.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _take_octs(p: ctypes.c_void_p, n: int) -> np.ndarray:
    L = lib()
    if n:
        buf = (ctypes.c_uint32 * (4 * n)).from_address(p.value)
        out = np.frombuffer(buf, dtype=np.uint32).reshape(n, 4).copy()
    else:
        out = np.zeros((0, 4), np.uint32)
    L.dgo_free(p)
    return out


class NoTermination(RuntimeError):
    """The reference's construction walk would loop forever on this input."""


def _check(rc: int, what: str):
    if rc == -4:
        raise NoTermination(f"oracle {what}: the reference walk does not terminate on this input")
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with code {rc}")


def quantize_sort(xyz: np.ndarray, max_depth: int = 30, glens=(1.0, 1.0, 1.0)) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    g = np.asarray(glens, np.float64)
    p = ctypes.c_void_p()
    _check(lib().dgo_quantize_sort(_ptr(xyz), xyz.shape[0], _ptr(g), max_depth, ctypes.byref(p)), "quantize_sort")
    return _take_octs(p, xyz.shape[0])


def points_to_octree(xyz: np.ndarray, max_depth: int = 30, max_pts: int = 1, glens=(1.0, 1.0, 1.0)) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    g = np.asarray(glens, np.float64)
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    _check(
        lib().dgo_points_to_octree(_ptr(xyz), xyz.shape[0], _ptr(g), max_depth, max_pts, ctypes.byref(p), ctypes.byref(n)),
        "points_to_octree",
    )
    return _take_octs(p, n.value)


def p2o_local(pts: np.ndarray, max_depth: int = 30, max_pts: int = 1) -> np.ndarray:
    pts = np.ascontiguousarray(pts, dtype=np.uint32).reshape(-1, 4)
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    _check(lib().dgo_p2o_local(_ptr(pts), pts.shape[0], max_depth, max_pts, ctypes.byref(p), ctypes.byref(n)), "p2o_local")
    return _take_octs(p, n.value)


def balance(octs: np.ndarray, max_depth: int = 30, inc_corner: bool = True) -> np.ndarray:
    octs = np.ascontiguousarray(octs, dtype=np.uint32).reshape(-1, 4)
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    _check(lib().dgo_balance_ex(_ptr(octs), octs.shape[0], max_depth, int(inc_corner), ctypes.byref(p),
                                ctypes.byref(n)), "balance")
    return _take_octs(p, n.value)


def coarsen(octs: np.ndarray, max_depth: int = 30) -> np.ndarray:
    octs = np.ascontiguousarray(octs, dtype=np.uint32).reshape(-1, 4)
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    _check(lib().dgo_coarsen(_ptr(octs), octs.shape[0], max_depth, ctypes.byref(p), ctypes.byref(n)), "coarsen")
    return _take_octs(p, n.value)


def complete(octs: np.ndarray, max_depth: int = 30, is_unique: bool = False, is_sorted: bool = False) -> np.ndarray:
    octs = np.ascontiguousarray(octs, dtype=np.uint32).reshape(-1, 4)
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    _check(lib().dgo_complete(_ptr(octs), octs.shape[0], max_depth, int(is_unique), int(is_sorted), ctypes.byref(p),
                              ctypes.byref(n)), "complete")
    return _take_octs(p, n.value)


def hilbert_sort(octs: np.ndarray, max_depth: int = 30) -> np.ndarray:
    a = np.array(octs, dtype=np.uint32).reshape(-1, 4)
    _check(lib().dgo_hilbert_sort(_ptr(a), a.shape[0], max_depth), "hilbert_sort")
    return a


def hilbert_states() -> int:
    return int(lib().dgo_hilbert_states())


def checks(octs: np.ndarray, max_depth: int = 30) -> dict:
    octs = np.ascontiguousarray(octs, dtype=np.uint32).reshape(-1, 4)
    L = lib()
    a = (_ptr(octs), octs.shape[0], max_depth)
    return {
        "sorted": bool(L.dgo_is_sorted_unique(*a)),
        "linear": bool(L.dgo_is_linear(*a)),
        "complete": bool(L.dgo_is_complete(*a)),
        "balanced": bool(L.dgo_is_balanced(*a)),
        "balanced_face_edge": bool(L.dgo_is_balanced_ex(*a, 0)),
    }


def fnv1a(octs: np.ndarray) -> int:
    octs = np.ascontiguousarray(octs, dtype=np.uint32).reshape(-1, 4)
    return int(lib().dgo_fnv1a(_ptr(octs), octs.shape[0]))


def etype_masks() -> np.ndarray:
    m = np.zeros(8 * 18, np.uint8)
    lib().dgo_etype_masks(_ptr(m))
    return m.reshape(8, 18)


def stencils():
    lap = np.zeros(8 * 18 * 64)
    mass = np.zeros(8 * 18 * 64)
    lib().dgo_stencils(_ptr(lap), _ptr(mass))
    return lap.reshape(8, 18, 8, 8), mass.reshape(8, 18, 8, 8)


def rmat_tables():
    r1 = np.zeros(8 * 8 * 18 * 64)
    r2 = np.zeros(8 * 18 * 64)
    lib().dgo_rmat_tables(_ptr(r1), _ptr(r2))
    return r1.reshape(8, 8, 18, 8, 8), r2.reshape(8, 18, 8, 8)


class DA:
    """Oracle DA: per-element child/hmask/etype/level/nodes and node coordinates."""

    def __init__(self, octs: np.ndarray, max_depth: int = 30):
        self.max_depth = max_depth
        octs = np.ascontiguousarray(octs, dtype=np.uint32).reshape(-1, 4)
        self._da = _DA()
        _check(lib().dgo_da_build(_ptr(octs), octs.shape[0], max_depth, ctypes.byref(self._da)), "da_build")
        ne, nn = self._da.n_elem, self._da.n_node

        def arr(p, n, dt):
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n else np.zeros(0, dt)

        self.n_elem, self.n_node = ne, nn
        self.child = arr(self._da.child, ne, np.uint8)
        self.hmask = arr(self._da.hmask, ne, np.uint8)
        self.etype = arr(self._da.etype, ne, np.uint8)
        self.level = arr(self._da.level, ne, np.uint8)
        self.nodes = arr(self._da.nodes, 8 * ne, np.uint32).reshape(ne, 8)
        self.node_xyz = arr(self._da.node_xyz, 3 * nn, np.uint32).reshape(nn, 3)

    def matvec(self, x: np.ndarray, lap_fac: float = 1.0, mass_fac: float = 1.0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        assert x.shape == (self.n_node,)
        y = np.zeros(self.n_node)
        _check(lib().dgo_matvec(ctypes.byref(self._da), self.max_depth, _ptr(x), _ptr(y), lap_fac, mass_fac), "matvec")
        return y

    def bdy(self) -> np.ndarray:
        dom = 1 << self.max_depth
        x = self.node_xyz
        return np.any((x == 0) | (x == dom), axis=1)

    def dirichlet_matvec(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n_node)
        _check(lib().dgo_dirichlet_matvec(ctypes.byref(self._da), self.max_depth, _ptr(x), _ptr(y)), "dirichlet_matvec")
        return y

    def dirichlet_diag(self) -> np.ndarray:
        d = np.zeros(self.n_node)
        _check(lib().dgo_dirichlet_diag(ctypes.byref(self._da), self.max_depth, _ptr(d)), "dirichlet_diag")
        return d

    def prolong_map(self, coarse_octs: np.ndarray, coarse: "DA"):
        """(ids, weights): 8 coarse nodes and weights per node of this (fine) mesh."""
        c = np.ascontiguousarray(coarse_octs, dtype=np.uint32).reshape(-1, 4)
        ids = np.zeros((self.n_node, 8), np.uint32)
        w = np.zeros((self.n_node, 8))
        _check(lib().dgo_prolong_map(ctypes.byref(self._da), _ptr(c), c.shape[0], ctypes.byref(coarse._da),
                                     self.max_depth, _ptr(ids), _ptr(w)), "prolong_map")
        return ids, w

    def __del__(self):
        try:
            lib().dgo_da_free(ctypes.byref(self._da))
        except Exception:
            pass


def element_matrices(da: "DA", lap_fac: float = 1.0, mass_fac: float = 1.0, coef=None) -> np.ndarray:
    """Per element the 8x8 (f1 L + f2 M) of odaJac.C:311-316 with
    f1 = lap h/2, f2 = mass h^3/8, h = 2^-level; lap/mass are the given
    factors or, with ``coef`` (n_elem x 2), each element's own
    (Jacobian2's matProp, omgJac.C:1666-1673)."""
    lap, mass = stencils()
    h = 1.0 / np.exp2(da.level.astype(np.float64))
    if coef is not None:
        c = np.asarray(coef, np.float64).reshape(-1, 2)
        lf, mf = c[:, 0], c[:, 1]
    else:
        lf, mf = lap_fac, mass_fac
    f1 = lf * h / 2.0
    f2 = mf * h * h * h / 8.0
    return f1[:, None, None] * lap[da.child, da.etype] + f2[:, None, None] * mass[da.child, da.etype]


def matvec_coef(da: "DA", coef, x: np.ndarray) -> np.ndarray:
    """Jacobian2MatMult (examples/src/backend/omgJac.C:1666-1735) on the
    oracle DA: y[idx[k]] += sum_j A_e[k][j] x[idx[j]]."""
    a = element_matrices(da, coef=coef)
    y = np.zeros(da.n_node)
    np.add.at(y, da.nodes, np.einsum("ekj,ej->ek", a, np.asarray(x, np.float64)[da.nodes]))
    return y


def diagonal(da: "DA", lap_fac: float = 1.0, mass_fac: float = 1.0, coef=None) -> np.ndarray:
    """Jacobian1MatGetDiagonal (odaJac.C:160-222) / Jacobian2MatGetDiagonal
    (omgJac.C:1641): the element matrices' diagonals summed per node."""
    a = element_matrices(da, lap_fac, mass_fac, coef)
    d = np.zeros(da.n_node)
    np.add.at(d, da.nodes, np.einsum("ekk->ek", a))
    return d


def assemble(da: "DA", lap_fac: float = 1.0, mass_fac: float = 1.0, dirichlet: bool = False, coef=None):
    """The assembled operator of the oracle DA as a scipy CSR matrix
    (duplicates summed): lap_fac K + mass_fac M, the records of
    CreateAndComputeFullJacobian1 (examples/src/backend/odaJac.C:470-535), or
    with ``dirichlet`` the Dirichlet K + M of ComputeDirichletJacobian
    (examples/src/backend/omgJac.C:383-490: interior rows and columns, the
    identity on boundary rows)."""
    import scipy.sparse as sp

    if dirichlet:
        lap_fac, mass_fac, coef = 1.0, 1.0, None
    a = element_matrices(da, lap_fac, mass_fac, coef)
    rows = np.broadcast_to(da.nodes[:, :, None], a.shape).ravel().astype(np.int64)
    cols = np.broadcast_to(da.nodes[:, None, :], a.shape).ravel().astype(np.int64)
    vals = a.ravel()
    n = da.n_node
    if dirichlet:
        b = da.bdy()
        keep = ~b[rows] & ~b[cols]
        ids = np.nonzero(b)[0]
        rows = np.concatenate([rows[keep], ids])
        cols = np.concatenate([cols[keep], ids])
        vals = np.concatenate([vals[keep], np.ones(len(ids))])
    m = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    m.sum_duplicates()
    m.sort_indices()
    return m

