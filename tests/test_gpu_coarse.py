"""The dense SPD inverse that the multigrid coarse solve applies
(dg_dense_spd_inverse): block Gauss-Jordan with the rank-64 trailing
updates on the tensor cores (3xTF32), checked against numpy in FP64 on a
well-conditioned matrix and on a graded-mesh-like Laplacian + mass operator."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spd_gram(n, rng):
    b = rng.standard_normal((n, n))
    return b @ b.T / n + np.eye(n)  # eigenvalues in about [1, 5]


def _laplacian_mass(n, rng):
    """A 3-D grid Laplacian (7-point, Dirichlet) on the first n cells of a
    cube plus a small mass term, symmetrically permuted: condition number in
    the hundreds, like the coarsest operator."""
    m = int(np.ceil(n ** (1 / 3)))
    idx = np.arange(m ** 3).reshape(m, m, m)
    a = np.zeros((m ** 3, m ** 3))
    for ax in range(3):
        lo = np.take(idx, range(m - 1), axis=ax).ravel()
        hi = np.take(idx, range(1, m), axis=ax).ravel()
        a[lo, hi] -= 1.0
        a[hi, lo] -= 1.0
    a[np.diag_indices_from(a)] = 6.0 + 0.01
    a = a[:n, :n]
    p = rng.permutation(n)
    return a[np.ix_(p, p)]


@pytest.mark.parametrize("n", [1, 5, 64, 65, 130, 257, 1000, 2600])
@pytest.mark.parametrize("kind", ["gram", "laplacian"])
def test_dense_spd_inverse(ctx, n, kind):
    import torch

    rng = np.random.Generator(np.random.PCG64(1000 + n))
    a = _spd_gram(n, rng) if kind == "gram" else _laplacian_mass(n, rng)
    x = torch.tensor(a, dtype=torch.float32, device="cuda")
    rc = ctx._L.dg_dense_spd_inverse(ctx.handle, ctypes.c_void_p(x.data_ptr()), n)
    assert rc == 0, ctx._L.dg_ctx_last_error(ctx.handle)
    xi = x.double().cpu().numpy()
    ref = np.linalg.inv(a)
    kappa = np.linalg.cond(a)
    # FP32 Gauss-Jordan: error about kappa * eps32 relative; the 3xTF32
    # updates add at most a few FP32 roundings per product
    rel = np.linalg.norm(xi - ref) / np.linalg.norm(ref)
    assert rel <= 2e-6 * max(kappa, 1.0), (rel, kappa)
    resid = np.abs(xi @ a - np.eye(n)).max()
    assert resid <= 2e-6 * max(kappa, 1.0) * 10, (resid, kappa)


def test_dense_spd_inverse_rejects(ctx):
    assert ctx._L.dg_dense_spd_inverse(ctx.handle, None, 4) != 0
    assert ctx._L.dg_dense_spd_inverse(ctx.handle, None, 0) == 0
