"""Global C0 solve (oracle restatement, FP64).

* gather / assemble with signs: AssemblyMapCG::v_GlobalToLocal / v_Assemble
  (MultiRegions/AssemblyMap/AssemblyMapCG.cpp:2853-2910) via Vmath::Gathr / Assmb
  (LibUtilities/BasicUtils/Vmath.cpp:756-840).
* operator: GlobalLinSysIterativeFull::v_DoMatrixMultiply (:215-257).
* Jacobi diagonal: PreconditionerDiagonal::DiagonalPreconditionerSum (:98-161),
  inverse applied by v_DoPreconditioner (:191-206).
* CG: NekLinSysIterCG::DoConjugateGradient (LibUtilities/LinearAlgebra/NekLinSysIterCG.cpp:104-263)
  with Set_Rhs_Magnitude's 1e-6 floor (NekLinSysIter.cpp:128-152).
* RHS: ContField::v_HelmSolve (MultiRegions/ContField.cpp:878-945): b = -Assemble(IProduct(f)).
The map is given as (l2g, sign, nglobal, ndir) arrays, Dirichlet ids first.
"""
import numpy as np

from . import ops


class Map:
    def __init__(self, l2g, sign, nglobal, ndir):
        self.l2g = np.asarray(l2g, dtype=np.int64)
        self.sign = np.asarray(sign, dtype=np.float64)
        self.nglobal, self.ndir = int(nglobal), int(ndir)

    @classmethod
    def of(cls, m):
        return cls(m.l2g, m.sign, m.nglobal, m.ndir)

    def gather(self, x):
        return self.sign * x[self.l2g]

    def assemble(self, loc):
        out = np.zeros(self.nglobal)
        np.add.at(out, self.l2g, self.sign * np.asarray(loc).reshape(-1))
        return out


def global_apply(basis, dim, jac, df, lam, amap, x, zero_dir=True):
    m = amap if isinstance(amap, Map) else Map.of(amap)
    xx = x.copy()
    if zero_dir:
        xx[:m.ndir] = 0.0
    return m.assemble(ops.helmholtz(basis, dim, jac, df, lam, m.gather(xx)).reshape(-1))


def jacobi_inverse(basis, dim, jac, df, lam, amap):
    m = amap if isinstance(amap, Map) else Map.of(amap)
    d = np.zeros(m.nglobal)
    np.add.at(d, m.l2g, m.sign * m.sign * ops.helmholtz_diag(basis, dim, jac, df, lam).reshape(-1))
    return 1.0 / d[m.ndir:]


def cg(apply_fn, dinv, rhs, ndir, tol=1e-9, max_iter=5000):
    """Returns (x, iterations, eps, rhs_mag); x has zeros on the Dirichlet part."""
    N = rhs.size
    nnd = N - ndir
    x = np.zeros(N)
    r = rhs[ndir:].copy()
    wA = np.zeros(N)
    p = np.zeros(nnd)
    q = np.zeros(nnd)
    eps = r @ r
    bb = rhs @ rhs
    rhs_mag = bb if bb > 1e-6 else 1.0
    tol = max(tol, 1e-16)
    if eps < tol * tol * rhs_mag:
        return x, 0, eps, rhs_mag
    wA[ndir:] = dinv * r
    sA = apply_fn(wA)
    rho = r @ wA[ndir:]
    mu = sA[ndir:] @ wA[ndir:]
    beta, alpha = 0.0, rho / mu
    iters, k = 1, 0
    while True:
        if k >= max_iter:
            raise RuntimeError("Exceeded maximum number of iterations")
        p = beta * p + wA[ndir:]
        q = beta * q + sA[ndir:]
        x[ndir:] += alpha * p
        r -= alpha * q
        wA[ndir:] = dinv * r
        sA = apply_fn(wA)
        rho_new = r @ wA[ndir:]
        mu = sA[ndir:] @ wA[ndir:]
        eps = r @ r
        iters += 1
        if eps < tol * tol * rhs_mag:
            break
        beta = rho_new / rho
        alpha = rho_new / (mu - rho_new * beta / alpha)
        rho = rho_new
        k += 1
    return x, iters, eps, rhs_mag


def solve(basis, dim, jac, df, lam, amap, rhs, tol=1e-9, max_iter=5000):
    m = amap if isinstance(amap, Map) else Map.of(amap)
    dinv = jacobi_inverse(basis, dim, jac, df, lam, m)
    return cg(lambda v: global_apply(basis, dim, jac, df, lam, m, v), dinv, rhs, m.ndir, tol, max_iter)


def helmsolve(basis, dim, jac, df, lam, amap, forcing, tol=1e-9, max_iter=5000, dirichlet=None):
    """HelmSolve (ContField.cpp:878-945): returns (local coefficients, iterations).
    dirichlet: the ndir Dirichlet global coefficients (None: homogeneous), lifted as the
    reference does: rhs_F -= (A x_D)_F, then x_D is the Dirichlet part of the result."""
    m = amap if isinstance(amap, Map) else Map.of(amap)
    rhs = -m.assemble(ops.iproduct(basis, dim, jac, forcing))
    xd = np.zeros(m.nglobal)
    if dirichlet is not None:
        xd[:m.ndir] = dirichlet
        rhs = rhs - global_apply(basis, dim, jac, df, lam, m, xd, zero_dir=False)
    x, it, _, _ = solve(basis, dim, jac, df, lam, m, rhs, tol, max_iter)
    x[:m.ndir] = xd[:m.ndir]
    return m.gather(x), it
