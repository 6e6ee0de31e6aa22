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


def cg(apply_fn, dinv, rhs, ndir, tol=1e-9, max_iter=5000, rhs_mag=None):
    """Returns (x, iterations, eps, rhs_mag); x has zeros on the Dirichlet part.
    rhs_mag: a magnitude set by the caller (GlobalLinSysIterative::Set_Rhs_Magnitude, as
    the static-condensation solve sets it); None: ||rhs||^2 with the 1e-6 floor."""
    N = rhs.size
    nnd = N - ndir
    x = np.zeros(N)
    r = rhs[ndir:].copy()
    wA = np.zeros(N)
    p = np.zeros(nnd)
    q = np.zeros(nnd)
    eps = r @ r
    if rhs_mag is None:
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


def solve_viscous(basis, dim, jac, df, amap, forcing, aii_dt, diff_coeff, dirichlet=None, tol=1e-9,
                  max_iter=5000):
    """VelocityCorrectionScheme_ROM::v_SolveViscous (solvers/IncNavierStokesSolver/
    EquationSystems/VelocityCorrectionScheme_ROM.cpp:1538-1567): per velocity field,
    lambda = 1 / aii_dt / diff_coeff[i], HelmSolve of forcing[i], then BwdTrans.
    Returns ([local coefficients], [physical values], [iterations])."""
    coeffs, phys, its = [], [], []
    for i, f in enumerate(forcing):
        lam = 1.0 / aii_dt / diff_coeff[i]
        d = None if dirichlet is None else dirichlet[i]
        c, it = helmsolve(basis, dim, jac, df, lam, amap, f, tol, max_iter, dirichlet=d)
        coeffs.append(c)
        phys.append(ops.bwdtrans(basis, dim, c).reshape(-1))
        its.append(it)
    return coeffs, phys, its


def solve_pressure(basis, dim, jac, df, amap, forcing, dirichlet=None, tol=1e-9, max_iter=5000):
    """VelocityCorrectionScheme_ROM::v_SolvePressure (:1522-1534): HelmSolve with
    lambda = 0 (the pressure Poisson equation). Returns (local coefficients, iterations)."""
    return helmsolve(basis, dim, jac, df, 0.0, amap, forcing, tol, max_iter, dirichlet=dirichlet)


# ---------------------------------------------------------------------------------
# Successive right-hand sides: projection onto previous solutions (Fischer 1998), as
# GlobalLinSysIterative::DoProjection / UpdateKnownSolutions / ResetKnownSolutionsToLatestOne
# (MultiRegions/GlobalLinSysIterative.cpp:156-482). nsucc > 0: A-conjugate basis of
# A-normalised solutions; nsucc < 0: the basis A x / ||A x|| (least squares in the
# Euclidean norm of the residual). The reference factorises the small symmetric
# coefficient matrix with Bunch-Kaufman (Lapack Dsptrf/Dsptrs); here an LDL^T without
# pivoting (the matrix is SPD with unit diagonal unless the basis is dependent, which
# the same tests reject).
# ---------------------------------------------------------------------------------
ZERO_TOL = 1.0e-12          # NekConstants::kNekZeroTol
SPARSE_NONZERO_TOL = 1e-16  # NekConstants::kNekSparseNonZeroTol


def ldlt_solve(M, y):
    """Solve M x = y by LDL^T without pivoting; returns None where a pivot is not positive."""
    n = M.shape[0]
    L = np.eye(n)
    d = np.zeros(n)
    for j in range(n):
        d[j] = M[j, j] - np.dot(L[j, :j] ** 2, d[:j])
        if not d[j] > 0.0:
            return None
        for i in range(j + 1, n):
            L[i, j] = (M[i, j] - np.dot(L[i, :j] * L[j, :j], d[:j])) / d[j]
    z = np.zeros(n)
    for i in range(n):
        z[i] = y[i] - np.dot(L[i, :i], z[:i])
    z /= d
    x = np.zeros(n)
    for i in range(n - 1, -1, -1):
        x[i] = z[i] - np.dot(L[i + 1:, i], x[i + 1:])
    return x


class SuccessiveRHS:
    def __init__(self, nsucc):
        self.aconj = nsucc > 0
        self.m = abs(int(nsucc))
        self.basis, self.sols = [], []
        self.M = np.zeros((0, 0))
        self.nprev = 0

    def _reset_to_latest(self):
        """ResetKnownSolutionsToLatestOne (:272-289)."""
        if self.nprev == 0:
            return -1
        latest = (self.nprev - 1 + self.m) % self.m
        self.basis, self.sols = [self.basis[latest]], [self.sols[latest]]
        self.M = np.ones((1, 1))  # the unit diagonal entry of the kept vector
        self.nprev = 1
        return latest

    def solve(self, apply_fn, dinv, rhs, ndir, tol=1e-9, max_iter=5000):
        """DoProjection (:156-266): returns (x, iterations of the CG on the projected rhs)."""
        if self.nprev == 0:
            x, it, _, _ = cg(apply_fn, dinv, rhs, ndir, tol, max_iter)
        else:
            b = rhs[ndir:]
            alpha = np.array([v @ b for v in self.basis])
            a = ldlt_solve(self.M, alpha)
            if a is None:
                latest = self._reset_to_latest()
                a = np.array([alpha[latest]])
            px = np.zeros(rhs.size)
            for ai, xi in zip(a, self.sols):
                px[ndir:] += ai * xi
            pb = np.zeros(rhs.size)
            pb[ndir:] = b - apply_fn(px)[ndir:]
            tmpx, it, _, _ = cg(apply_fn, dinv, pb, ndir, tol, max_iter)
            x = np.zeros(rhs.size)
            x[ndir:] = tmpx[ndir:] + px[ndir:]
        if it:
            self._update(apply_fn, x, ndir)
        return x, it

    def _update(self, apply_fn, newx, ndir):
        """UpdateKnownSolutions (:295-482)."""
        m = self.m
        insert = self.nprev % m
        full = len(self.basis) == m
        ax = apply_fn(newx)[ndir:]
        xb = newx[ndir:]
        new_basis = xb if self.aconj else ax
        sol_norm = new_basis @ ax
        if sol_norm < 22.2 * SPARSE_NONZERO_TOL:
            return
        axn = ax / np.sqrt(sol_norm)
        y = np.array([self.basis[i] @ axn for i in range(len(self.basis)) if i != insert])
        if full and m > 1:
            keep = [i for i in range(m) if i != insert]
            tilM = self.M[np.ix_(keep, keep)]
        elif not full and len(self.basis):
            tilM = self.M.copy()
        else:
            tilM = np.zeros((0, 0))
        ok = True
        inv_y = np.zeros(y.size)
        if y.size:
            s = ldlt_solve(tilM, y)
            ok = s is not None
            if ok:
                inv_y = s
        if not ok:
            latest = self._reset_to_latest()
            y = np.array([y[latest - (latest > insert)]])
            inv_y = y.copy()
            insert = self.nprev % m
            full = len(self.basis) == m
        residual = 1.0 - float(np.dot(y[:len(self.basis) - full], inv_y[:len(self.basis) - full]))
        if residual < 10.0 * ZERO_TOL:
            return
        if full:
            newM = self.M.copy()
            newM[insert, insert] = 1.0
            for i in range(m):
                if i == insert:
                    continue
                newM[insert, i] = newM[i, insert] = y[i - (i > insert)]
        else:
            k = len(self.basis)
            newM = np.zeros((k + 1, k + 1))
            newM[:k, :k] = self.M
            newM[insert, insert] = 1.0
            for i in range(k):
                newM[insert, i] = newM[i, insert] = y[i]
        if ldlt_solve(newM, np.ones(newM.shape[0])) is None:
            return
        xs = xb / np.sqrt(sol_norm)
        if len(self.basis) < m:
            self.basis.append(None)
            self.sols.append(None)
        self.sols[insert] = xs
        self.basis[insert] = xs if self.aconj else axn
        self.M = newM
        self.nprev += 1
