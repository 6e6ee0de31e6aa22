"""Variable-coefficient Helmholtz and the adjoint gradient (oracle restatement, FP64).

Operator: A(kappa) u = lambda M u + L_kappa u with L_kappa = sum_ab (d_a phi, kappa g^{ab} d_b u)_J,
the isotropic case of StdRegions/StdExpansion.cpp:664-717 (LaplacianMatrixOp_MatFree with
eVarCoeffD00 = eVarCoeffD11 [= D22] = kappa at the quadrature points).
Misfit: J(kappa) = sum_q Jw_q (u(x_q) - u_t(x_q))^2 (quadrature of ||u - u_t||^2).
Adjoint (no counterpart in the reference): A psi = dJ/du, and
  dJ/dkappa_q = -Jw_q grad psi(x_q) . grad u(x_q).
"""
import numpy as np

from . import ops
from . import solve as osolve


def global_apply_kappa(basis, dim, jac, df, lam, kappa, m, x):
    xx = x.copy()
    xx[:m.ndir] = 0.0
    return m.assemble(ops.helmholtz_varcoeff(basis, dim, jac, df, lam, kappa, m.gather(xx)).reshape(-1))


def jacobi_inverse_kappa(basis, dim, jac, df, lam, kappa, m):
    """Diagonal of A(kappa) by probing the element operator with unit vectors per mode."""
    E = np.asarray(jac).shape[0]
    nm = basis.n ** dim
    d = np.zeros((E, nm))
    for k in range(nm):
        u = np.zeros((E, nm))
        u[:, k] = 1.0
        d[:, k] = ops.helmholtz_varcoeff(basis, dim, jac, df, lam, kappa, u.reshape(-1)).reshape(E, nm)[:, k]
    g = np.zeros(m.nglobal)
    np.add.at(g, m.l2g, d.reshape(-1))
    return 1.0 / g[m.ndir:]


def solve_kappa(basis, dim, jac, df, lam, kappa, m, rhs, tol=1e-12, max_iter=5000):
    dinv = jacobi_inverse_kappa(basis, dim, jac, df, lam, kappa, m)
    x, it, _, _ = osolve.cg(lambda v: global_apply_kappa(basis, dim, jac, df, lam, kappa, m, v), dinv, rhs, m.ndir,
                            tol, max_iter)
    return x, it


def misfit(basis, dim, jac, m, x, u_target_phys):
    """J and dJ/dx (global, zero on Dirichlet dofs)."""
    E = np.asarray(jac).shape[0]
    xx = x.copy()
    xx[:m.ndir] = 0.0
    u = ops.bwdtrans(basis, dim, m.gather(xx)).reshape(E, -1)
    diff = u - u_target_phys.reshape(E, -1)
    w = np.outer(basis.w, basis.w).reshape(-1) if dim == 2 else np.einsum(
        "k,j,i->kji", basis.w, basis.w, basis.w).reshape(-1)
    Jw = np.asarray(jac).reshape(E, -1) * w[None]
    J = float(np.sum(Jw * diff * diff))
    g = 2.0 * m.assemble(ops.iproduct(basis, dim, jac, diff).reshape(-1))
    g[:m.ndir] = 0.0
    return J, g


def kappa_gradient(basis, dim, jac, df, m, x, psi):
    """dJ/dkappa_q = -Jw_q grad psi . grad u at every quadrature point, shape (E, Q^d)."""
    E = np.asarray(jac).shape[0]
    xx, pp = x.copy(), psi.copy()
    xx[:m.ndir] = 0.0
    pp[:m.ndir] = 0.0
    du = ops.physderiv(basis, dim, df, ops.bwdtrans(basis, dim, m.gather(xx)).reshape(-1))
    dp = ops.physderiv(basis, dim, df, ops.bwdtrans(basis, dim, m.gather(pp)).reshape(-1))
    w = np.outer(basis.w, basis.w).reshape(-1) if dim == 2 else np.einsum(
        "k,j,i->kji", basis.w, basis.w, basis.w).reshape(-1)
    Jw = np.asarray(jac).reshape(E, -1) * w[None]
    return -Jw * sum(a * b for a, b in zip(du, dp))


def objective_and_gradient(basis, dim, jac, df, lam, kappa, m, rhs, u_target_phys, tol=1e-13):
    x, _ = solve_kappa(basis, dim, jac, df, lam, kappa, m, rhs, tol)
    J, g = misfit(basis, dim, jac, m, x, u_target_phys)
    psi, _ = solve_kappa(basis, dim, jac, df, lam, kappa, m, g, tol)
    return J, kappa_gradient(basis, dim, jac, df, m, x, psi), x


def smooth_field(X, seed, nmodes=8):
    """Seeded smooth field: sum of 8 Fourier modes, normalised to max |g| <= 1."""
    rng = np.random.default_rng(seed)
    g = np.zeros_like(X[0])
    for _ in range(nmodes):
        kx, ky = rng.integers(1, 4, size=2)
        a = rng.uniform(-1, 1)
        px, py = rng.uniform(0, 2 * np.pi, size=2)
        g = g + a * np.sin(np.pi * kx * X[0] + px) * np.sin(np.pi * ky * X[1] + py)
    return g / max(np.max(np.abs(g)), 1e-300)
