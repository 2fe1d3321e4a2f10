"""CPU multigrid oracle: the reference's DAMG hierarchy and PCG + V-cycle solve.

TEST INFRASTRUCTURE ONLY (checker for dendro_gb300.MultiGrid).

Levels follow src/omg/blockDiag.cpp:1384-1425: coarsenOctree
(src/coarsen.cpp:53) then balanceOctree, repeated until a level holds at most
``max_coarse`` elements.  The operator is DirichletJacobianMatMult
(examples/src/backend/omgJac.C:958), the transfers are the transpose pair
of restrictMatVecType1 (src/omg/restrictMatVec.cpp:74-146).  The solver is
the standard preconditioned CG with one multiplicative V-cycle per
iteration, damped-Jacobi smoothing and an exact coarsest solve -- the
algorithms PETSc's KSPCG / PCMG / Richardson+Jacobi / LU apply for the
reference (bin/options:48-206).  PETSc itself is not available, so this
part is a restatement of those published algorithms, not pinned to PETSc's
own iterates.
"""
from __future__ import annotations

import numpy as np

from . import dg_oracle as O


class OracleMG:
    def __init__(self, bal: np.ndarray, max_depth: int = 30, max_coarse: int = 4096, omega: float = 0.667,
                 nu_pre: int = 2, nu_post: int = 2):
        self.D = max_depth
        self.omega, self.nu_pre, self.nu_post = omega, nu_pre, nu_post
        octs = [np.ascontiguousarray(bal, np.uint32)]
        while len(octs[-1]) > max_coarse:
            c = O.coarsen(octs[-1], max_depth)
            if len(c) == len(octs[-1]):
                break
            octs.append(O.balance(c, max_depth))
        self.octs = octs
        self.das = [O.DA(o, max_depth) for o in octs]
        self.dinv = [1.0 / da.dirichlet_diag() for da in self.das]
        self.pmaps = [self.das[l].prolong_map(octs[l + 1], self.das[l + 1]) for l in range(len(octs) - 1)]
        cda = self.das[-1]
        n = cda.n_node
        A = np.zeros((n, n))
        for i in range(n):
            e = np.zeros(n)
            e[i] = 1.0
            A[:, i] = cda.dirichlet_matvec(e)
        self.cinv = np.linalg.inv(A)

    @property
    def n_levels(self):
        return len(self.octs)

    def matvec(self, l, x):
        return self.das[l].dirichlet_matvec(x)

    def prolong(self, l, xc):
        ids, w = self.pmaps[l]
        return (w * xc[ids]).sum(axis=1)

    def restrict(self, l, rf):
        ids, w = self.pmaps[l]
        bc = np.zeros(self.das[l + 1].n_node)
        np.add.at(bc, ids.ravel(), (w * rf[:, None]).ravel())
        return bc

    def vcycle(self, l, b):
        if l == self.n_levels - 1:
            return self.cinv @ b
        om, dinv = self.omega, self.dinv[l]
        x = np.zeros_like(b)
        for it in range(self.nu_pre):
            x = om * dinv * b if it == 0 else x + om * dinv * (b - self.matvec(l, x))
        r = b - self.matvec(l, x)
        x = x + self.prolong(l, self.vcycle(l + 1, self.restrict(l, r)))
        for _ in range(self.nu_post):
            x = x + om * dinv * (b - self.matvec(l, x))
        return x

    def rhs(self, f):
        b = self.das[0].matvec(f, 0.0, 1.0)
        b[self.das[0].bdy()] = 0.0
        return b

    def solve(self, b, rtol=1e-8, maxit=200):
        x = np.zeros_like(b)
        r = b.copy()
        bn = np.linalg.norm(b)
        z = self.vcycle(0, r)
        p = z.copy()
        rz = r @ z
        it = 0
        for it in range(1, maxit + 1):
            q = self.matvec(0, p)
            a = rz / (p @ q)
            x += a * p
            r -= a * q
            if np.linalg.norm(r) / bn <= rtol:
                break
            z = self.vcycle(0, r)
            rzn = r @ z
            p = z + (rzn / rz) * p
            rz = rzn
        relres = np.linalg.norm(b - self.matvec(0, x)) / bn
        return x, it, relres
