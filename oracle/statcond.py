"""Static condensation of the C0 Helmholtz system (oracle restatement, FP64).

Follows
  * GlobalLinSysStaticCond::v_Solve (MultiRegions/GlobalLinSysStaticCond.cpp:104-238):
    F_bnd = local boundary forcing, F_int = local interior forcing;
    F_bnd -= BinvD F_int; F_bnd -= S V_bnd (V_bnd: the boundary values already in the
    output, Dirichlet data and initial guess); solve the assembled boundary system for
    the perturbation; V_bnd += perturbation; V_int = invD (F_int - C V_bnd);
  * the element blocks of StdExpansion's static condensation (m_schurCompl = A_bb -
    A_bi A_ii^-1 A_ib, m_BinvD = A_bi A_ii^-1, m_C = A_ib, m_invD = A_ii^-1) of the dense
    element Helmholtz matrices;
  * GlobalLinSysIterativeStaticCond::v_PreSolve (GlobalLinSysIterativeStaticCond.cpp:431-460):
    the CG's rhs magnitude is ||AssembleBnd(F_bnd)||^2 of the boundary forcing before
    condensation (1e-6 floor; smoothed 0.9 / 0.1 with the previous solve's value on later
    solves of the same system);
  * PreconditionerDiagonal::StaticCondDiagonalPreconditionerSum
    (MultiRegions/PreconditionerDiagonal.cpp:164-189): the Jacobi preconditioner is the
    inverse of the assembled diagonal of the element Schur complements;
  * v_DoMatrixMultiply (GlobalLinSysIterativeStaticCond.cpp:392-424): GlobalToLocalBnd,
    the element Schur complements, AssembleBnd.
Boundary modes of ModifiedA quads / hexes: those with any modal index below 2 (vertex,
edge and face modes); interior: all indices >= 2. Element-interior modes are private to
their element, so the boundary numbering compacts the global ids of boundary modes,
keeping the Dirichlet ids (numbered first) first.
"""
import numpy as np

from . import ops
from .solve import cg


def boundary_mask(n, dim):
    idx = np.indices((n,) * dim).reshape(dim, -1)  # [(r,) q, p] with p fastest
    return np.any(idx < 2, axis=0)


def element_matrices(basis, dim, jac, df, lam):
    """Dense element Helmholtz matrices A[e][i, j] = (operator applied to unit mode j)_i."""
    nm = basis.n ** dim
    E = np.asarray(jac).reshape(-1).size // (basis.Q ** dim)  # deformed (per-point) geometry
    A = np.zeros((E, nm, nm))
    for j in range(nm):
        u = np.zeros((E, nm))
        u[:, j] = 1.0
        A[:, :, j] = ops.helmholtz(basis, dim, jac, df, lam, u.reshape(-1)).reshape(E, nm)
    return A


class StaticCond:
    def __init__(self, basis, dim, jac, df, lam, amap):
        self.dim, self.n = dim, basis.n
        nm = basis.n ** dim
        self.bmask = boundary_mask(basis.n, dim)
        self.bi = np.flatnonzero(self.bmask)
        self.ii = np.flatnonzero(~self.bmask)
        A = element_matrices(basis, dim, jac, df, lam)
        self.E = A.shape[0]
        Abb = A[:, self.bi][:, :, self.bi]
        Abi = A[:, self.bi][:, :, self.ii]
        Aib = A[:, self.ii][:, :, self.bi]
        Aii = A[:, self.ii][:, :, self.ii]
        self.invD = np.linalg.inv(Aii)
        self.BinvD = Abi @ self.invD
        self.C = Aib
        self.S = Abb - self.BinvD @ Aib
        l2g = amap.l2g.reshape(self.E, nm)
        sign = amap.sign.reshape(self.E, nm)
        gb = l2g[:, self.bi]
        ids = np.unique(gb)  # sorted: the Dirichlet ids (< ndir) stay first
        self.bl2g = np.searchsorted(ids, gb)
        self.bsign = sign[:, self.bi]
        self.nb_glob = ids.size
        self.ndir = int(np.sum(ids < amap.ndir))
        self.gid = ids  # boundary id -> full global id
        d = np.zeros(self.nb_glob)
        np.add.at(d, self.bl2g, self.bsign ** 2 * np.einsum("eii->ei", self.S))
        self.dinv = 1.0 / d[self.ndir:]
        self.rhs_mag = None

    def assemble_bnd(self, loc):
        out = np.zeros(self.nb_glob)
        np.add.at(out, self.bl2g, self.bsign * loc)
        return out

    def global_to_local_bnd(self, x):
        return self.bsign * x[self.bl2g]

    def apply(self, x):
        """v_DoMatrixMultiply: Dirichlet entries of x read as they are (the CG's vectors
        carry zeros there)."""
        xl = self.global_to_local_bnd(x)
        return self.assemble_bnd(np.einsum("eij,ej->ei", self.S, xl))

    def solve(self, loc_rhs, loc_inout, tol=1e-9, max_iter=5000):
        """GlobalLinSysStaticCond::v_Solve: returns (local solution, CG iterations)."""
        E, nm = self.E, self.n ** self.dim
        F = np.asarray(loc_rhs).reshape(E, nm)
        V = np.asarray(loc_inout, dtype=float).reshape(E, nm).copy()
        F_int = F[:, self.ii]
        F_bnd = F[:, self.bi].copy()
        V_bnd = V[:, self.bi].copy()
        bb = self.assemble_bnd(F_bnd)
        new_mag = bb @ bb
        new_mag = new_mag if new_mag > 1e-6 else 1.0
        self.rhs_mag = new_mag if self.rhs_mag is None else 0.9 * self.rhs_mag + 0.1 * new_mag
        F_bnd -= np.einsum("eij,ej->ei", self.BinvD, F_int)
        F_bnd -= np.einsum("eij,ej->ei", self.S, V_bnd)
        Fg = self.assemble_bnd(F_bnd)
        pert, it, _, _ = cg(self.apply, self.dinv, Fg, self.ndir, tol, max_iter, rhs_mag=self.rhs_mag)
        V_bnd += self.global_to_local_bnd(pert)
        V_int = np.einsum("eij,ej->ei", self.invD, F_int - np.einsum("eij,ej->ei", self.C, V_bnd))
        out = np.zeros((E, nm))
        out[:, self.bi] = V_bnd
        out[:, self.ii] = V_int
        return out.reshape(-1), it


def helmsolve(basis, dim, jac, df, lam, amap, forcing, tol=1e-9, max_iter=5000, dirichlet=None, sc=None):
    """ContField::v_HelmSolve with the static-condensation solve: returns (local
    coefficients, iterations, the StaticCond object)."""
    sc = sc or StaticCond(basis, dim, jac, df, lam, amap)
    E, nm = sc.E, basis.n ** dim
    loc_rhs = -ops.iproduct(basis, dim, jac, forcing).reshape(-1)
    inout = np.zeros(E * nm)
    if dirichlet is not None:
        xg = np.zeros(amap.nglobal)
        xg[:amap.ndir] = dirichlet
        inout = (amap.sign * xg[amap.l2g]).reshape(-1)
    x, it = sc.solve(loc_rhs, inout, tol, max_iter)
    return x, it, sc
