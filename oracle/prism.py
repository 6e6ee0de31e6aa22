"""Prism element operators (oracle restatement, FP64). Test infrastructure only.

Expansion (the default keys of SpatialDomains/MeshGraph.cpp:1011-1045):
  directions 0, 1  eModified_A, n modes on Q0 = Q1 = n + 1 Gauss-Lobatto-Legendre points
  direction 2      eModified_B on Q2 = n Gauss-Radau-Jacobi points (alpha 1, beta 0), rows
                   (p, r) of the (eta0, eta2) triangle
Modes m(p, q, r): r fastest, then q, then p, with p, q < n and r < n - p. Physical layout
u[e, (k Q1 + j) Q0 + i]. Geometry: ``jac`` (E,) or (E, nq); ``df`` (9, E) or (9, E nq).

Operators restate the MatrixFree prism kernels with CORRECT = true:
  bwdtrans   MatrixFreeOps/BwdTransKernels.hpp:224-300 (BwdTransPrismKernel): the modes
             (0, q, 1) of the singular edge also carry B0[1] in direction 0
  iproduct   MatrixFreeOps/IProductKernels.hpp:316-449 (IProductPrismKernel), Gauss-Radau
             weights times 0.5 (MatrixFreeOps/Operator.hpp:245-248)
  physderiv  MatrixFreeOps/PhysDerivKernels.hpp:376-470 (PhysDerivPrismKernel)
  helmholtz  MatrixFreeOps/Helmholtz.h:1003-1030, 1291-1440 (HelmholtzPrismImpl)
  iproduct_deriv  MatrixFreeOps/IProductWRTDerivBase.h:1660-1760
"""
import numpy as np

from . import polylib
from .basis import Basis1D
from .tet import modB_rows
from .tri import lagrange_d, radau_m


def prism_modes(n):
    return [(p, q, r) for p in range(n) for q in range(n) for r in range(n - p)]


def pr_index(n, p, r):
    return sum(n - pp for pp in range(p)) + r


class PrismBasis:
    def __init__(self, n):
        self.n = n
        self.Q0 = self.Q1 = n + 1
        self.Q2 = n
        a = Basis1D(n, n + 1)
        self.z0, self.w0, self.D0 = a.z, a.w, a.D
        self.B0, self.DB0, self.D0_2 = a.B2, a.DB2, a.D2
        self.z2, self.w2 = radau_m(n)
        self.D2 = lagrange_d(self.z2)
        self.D2_2 = self.D2.reshape(n, n).T
        self.B2 = modB_rows(n, self.z2)                   # [pr, k]
        self.DB2 = (self.D2_2 @ self.B2.T).T
        self.w2h = 0.5 * self.w2
        self.modes = prism_modes(n)
        self.nc = len(self.modes)
        self.pr_of = np.array([pr_index(n, p, r) for (p, q, r) in self.modes])
        self.p_of = np.array([p for (p, q, r) in self.modes])
        self.q_of = np.array([q for (p, q, r) in self.modes])
        self.nq = self.Q0 * self.Q1 * self.Q2

    def weights(self):
        return (self.w2h[:, None, None] * self.w0[None, :, None] * self.w0[None, None, :]).reshape(-1)


def _pts(a, E, nq):
    a = np.asarray(a, dtype=np.float64)
    if a.size == E:
        return np.repeat(a.reshape(E, 1), nq, axis=1)
    return a.reshape(E, nq)


def bwdtrans(pb, coeffs):
    n = pb.n
    c = np.asarray(coeffs, dtype=np.float64).reshape(-1, pb.nc)
    E = c.shape[0]
    # u[k, j, i] = sum_m B0[p, i] B0[q, j] B2[pr, k] c[m]
    u = np.einsum("mi,mj,mk,em->ekji", pb.B0[pb.p_of], pb.B0[pb.q_of], pb.B2[pb.pr_of], c)
    for q in range(n):   # singular edge: c[(0, q, 1)] B2[1] B0[q] B0[1]
        u += c[:, q * n + 1][:, None, None, None] * np.einsum("k,j,i->kji", pb.B2[1], pb.B0[q], pb.B0[1])[None]
    return u.reshape(E, pb.nq)


def iproduct_tables(pb, A0, A1, A2, fw):
    n = pb.n
    E = fw.shape[0]
    f = fw.reshape(E, pb.Q2, pb.Q1, pb.Q0)
    out = np.einsum("mi,mj,mk,ekji->em", A0[pb.p_of], A1[pb.q_of], A2[pb.pr_of], f)
    for q in range(n):
        out[:, q * n + 1] += np.einsum("ekji,k,j,i->e", f, A2[1], A1[q], A0[1])
    return out


def iproduct(pb, jac, phys):
    phys = np.asarray(phys, dtype=np.float64).reshape(-1, pb.nq)
    E = phys.shape[0]
    return iproduct_tables(pb, pb.B0, pb.B0, pb.B2, phys * _pts(jac, E, pb.nq) * pb.weights()[None])


def collapsed_derivs(pb, phys):
    u = np.asarray(phys, dtype=np.float64).reshape(-1, pb.Q2, pb.Q1, pb.Q0)
    E = u.shape[0]
    d0 = np.einsum("ab,ekjb->ekja", pb.D0_2, u)
    d1 = np.einsum("ab,ekbi->ekai", pb.D0_2, u)
    d2 = np.einsum("ab,ebji->eaji", pb.D2_2, u)
    return [d.reshape(E, -1) for d in (d0, d1, d2)]


def _factors(pb):
    """Per point: h0 = (1 + z0)/2, h1 = 2/(1 - z2)."""
    H0 = np.tile(0.5 * (1 + pb.z0), pb.Q1 * pb.Q2)[None]
    H1 = np.repeat(2.0 / (1 - pb.z2), pb.Q0 * pb.Q1)[None]
    return H0, H1


def xi_derivs(pb, phys):
    d0, d1, d2 = collapsed_derivs(pb, phys)
    H0, H1 = _factors(pb)
    x0 = H1 * d0
    return x0, d1, d2 + H0 * x0


def physderiv(pb, df, phys):
    u = np.asarray(phys, dtype=np.float64).reshape(-1, pb.nq)
    E = u.shape[0]
    x = xi_derivs(pb, u)
    f = [_pts(df[k], E, pb.nq) for k in range(9)]
    return [sum(f[c * 3 + j] * x[j] for j in range(3)) for c in range(3)]


def helmholtz(pb, jac, df, lam, coeffs):
    """lambda M u + L u, composed as HelmholtzPrismImpl."""
    c = np.asarray(coeffs, dtype=np.float64).reshape(-1, pb.nc)
    E = c.shape[0]
    nq = pb.nq
    J = _pts(jac, E, nq)
    W = pb.weights()[None]
    bwd = bwdtrans(pb, c)
    out = lam * iproduct_tables(pb, pb.B0, pb.B0, pb.B2, bwd * J * W)
    d0, d1, d2 = collapsed_derivs(pb, bwd)
    H0, H1 = _factors(pb)
    f = [_pts(df[k], E, nq) for k in range(9)]
    a = [H1 * (H0 * f[3 * cc + 2] + f[3 * cc]) for cc in range(3)]
    b = [f[3 * cc + 1] for cc in range(3)]
    e = [f[3 * cc + 2] for cc in range(3)]
    g0 = sum(x * x for x in a)
    g1 = sum(x * x for x in b)
    g2 = sum(x * x for x in e)
    g3 = sum(x * y for x, y in zip(a, b))
    g4 = sum(x * y for x, y in zip(a, e))
    g5 = sum(x * y for x, y in zip(b, e))
    t0 = g0 * d0 + g3 * d1 + g4 * d2
    t1 = g3 * d0 + g1 * d1 + g5 * d2
    t2 = g4 * d0 + g5 * d1 + g2 * d2
    out = out + iproduct_tables(pb, pb.DB0, pb.B0, pb.B2, t0 * J * W)
    out = out + iproduct_tables(pb, pb.B0, pb.DB0, pb.B2, t1 * J * W)
    out = out + iproduct_tables(pb, pb.B0, pb.B0, pb.DB2, t2 * J * W)
    return out


def iproduct_deriv(pb, jac, df, comps):
    cs = [np.asarray(x, dtype=np.float64).reshape(-1, pb.nq) for x in comps]
    E = cs[0].shape[0]
    J = _pts(jac, E, pb.nq)
    W = pb.weights()[None]
    f = [_pts(df[k], E, pb.nq) for k in range(9)]
    t = [sum(f[3 * c + j] * cs[c] for c in range(3)) for j in range(3)]
    H0, H1 = _factors(pb)
    a = H1 * (t[0] + H0 * t[2])
    return (iproduct_tables(pb, pb.DB0, pb.B0, pb.B2, a * J * W) +
            iproduct_tables(pb, pb.B0, pb.DB0, pb.B2, t[1] * J * W) +
            iproduct_tables(pb, pb.B0, pb.B0, pb.DB2, t[2] * J * W))


def helmholtz_diag(pb, E, jac, df, lam):
    d = np.zeros((E, pb.nc))
    for m in range(pb.nc):
        u = np.zeros((E, pb.nc))
        u[:, m] = 1.0
        d[:, m] = helmholtz(pb, jac, df, lam, u)[:, m]
    return d


def geom_factors(pb, X):
    X = np.asarray(X, dtype=np.float64)
    E = X.shape[1]
    dx = np.stack([np.stack(xi_derivs(pb, X[c])) for c in range(3)])
    M = np.moveaxis(dx, (0, 1), (-2, -1))
    J = np.linalg.det(M)
    inv = np.linalg.inv(M)
    df = np.stack([inv[..., j, c] for c in range(3) for j in range(3)]).reshape(9, E * pb.nq)
    return J, df


def modal_values(n, xi0, xi1, xi2):
    """phi_m at reference points with xi2 < 1: (npts, nc), the modes (0, q, 1) with their
    singular-edge term (no eta0 factor)."""
    xi0, xi1, xi2 = (np.asarray(a, dtype=np.float64) for a in (xi0, xi1, xi2))
    e0 = 2 * (1 + xi0) / (1 - xi2) - 1
    shape = np.broadcast(e0, xi1, xi2).shape

    def modA(p, x):
        if p == 0:
            return 0.5 * (1 - x)
        if p == 1:
            return 0.5 * (1 + x)
        return 0.25 * (1 - x) * (1 + x) * polylib.jacobi(p - 2, 1.0, 1.0, x)
    B2 = modB_rows(n, np.broadcast_to(xi2, shape).reshape(-1)).reshape((-1,) + shape)
    cols = []
    for (p, q, r) in prism_modes(n):
        a = np.ones(shape) if (p == 0 and r == 1) else modA(p, e0)
        cols.append(a * modA(q, xi1) * B2[pr_index(n, p, r)])
    return np.stack(cols, axis=-1)
