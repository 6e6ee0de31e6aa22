"""Pyramid element operators (oracle restatement, FP64). Test infrastructure only.

Expansion (the default keys of SpatialDomains/MeshGraph.cpp:1719-1745):
  directions 0, 1  eModified_A, n modes on Q0 = Q1 = n + 1 Gauss-Lobatto-Legendre points
  direction 2      eModifiedPyr_C on Q2 = n Gauss-Radau-Jacobi points (alpha 2, beta 0)
                   (LibUtilities/Foundations/Basis.cpp:568-672): the row of mode (p, q, r) is
                   the eModified_B row (max(p, q), r) when min(p, q) <= 1, otherwise
                   ((1-z)/2)^(p+q-2) for r = 0 and ((1-z)/2)^(p+q-2) (1+z)/2 P_{r-1}^{(2p+2q-3,1)}
Modes m(p, q, r): r fastest, then q, then p, with r < n - max(p, q)
(n (n+1) (2n+1) / 6 of them). Physical layout u[e, (k Q1 + j) Q0 + i].

Operators restate the MatrixFree pyramid kernels with CORRECT = true (the top vertex):
  bwdtrans   MatrixFreeOps/BwdTransKernels.hpp:128-222 (BwdTransPyrKernel)
  iproduct   MatrixFreeOps/IProductKernels.hpp:452-600 (IProductPyrKernel), Gauss-Radau
             weights times 0.25 (MatrixFreeOps/Operator.hpp:249-251)
  physderiv  MatrixFreeOps/PhysDerivKernels.hpp:463-552 (PhysDerivPyrKernel)
  helmholtz  MatrixFreeOps/Helmholtz.h:1480-1510, 1770-1960 (HelmholtzPyrImpl)
  iproduct_deriv  MatrixFreeOps/IProductWRTDerivBase.h:2070-2200
"""
import numpy as np

from . import polylib
from .basis import Basis1D
from .tet import modB_rows, pair_index, radau_m
from .tri import lagrange_d


def pyr_modes(n):
    return [(p, q, r) for p in range(n) for q in range(n) for r in range(n - max(p, q))]


def pyrC_rows(n, z):
    z = np.asarray(z, dtype=np.float64)
    b = modB_rows(n, z)
    lo, hi = 0.5 * (1 - z), 0.5 * (1 + z)
    rows = []
    for (p, q, r) in pyr_modes(n):
        if min(p, q) <= 1:
            rows.append(b[pair_index(n, max(p, q), r)])
        elif r == 0:
            rows.append(lo ** (p + q - 2))
        else:
            rows.append(lo ** (p + q - 2) * hi * polylib.jacobi(r - 1, 2.0 * p + 2.0 * q - 3.0, 1.0, z))
    return np.array(rows)


class PyrBasis:
    def __init__(self, n):
        self.n = n
        self.Q0 = self.Q1 = n + 1
        self.Q2 = n
        a = Basis1D(n, n + 1)
        self.z0, self.w0, self.D0 = a.z, a.w, a.D
        self.B0, self.DB0, self.D0_2 = a.B2, a.DB2, a.D2
        self.z2, self.w2 = radau_m(n, 2)
        self.D2 = lagrange_d(self.z2)
        self.D2_2 = self.D2.reshape(n, n).T
        self.B2 = pyrC_rows(n, self.z2)
        self.DB2 = (self.D2_2 @ self.B2.T).T
        self.w2h = 0.25 * self.w2
        self.modes = pyr_modes(n)
        self.nc = len(self.modes)
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


def bwdtrans(yb, coeffs):
    c = np.asarray(coeffs, dtype=np.float64).reshape(-1, yb.nc)
    E = c.shape[0]
    B0 = yb.B0
    u = np.einsum("mi,mj,mk,em->ekji", B0[yb.p_of], B0[yb.q_of], yb.B2, c)
    top = np.outer(B0[1], B0[0]) + np.outer(B0[0], B0[1]) + np.outer(B0[1], B0[1])   # [j, i]
    u += c[:, 1][:, None, None, None] * yb.B2[1][None, :, None, None] * top[None, None]
    return u.reshape(E, yb.nq)


def iproduct_tables(yb, A0, A1, A2, fw):
    E = fw.shape[0]
    f = fw.reshape(E, yb.Q2, yb.Q1, yb.Q0)
    out = np.einsum("mi,mj,mk,ekji->em", A0[yb.p_of], A1[yb.q_of], A2, f)
    top = np.outer(A1[1], A0[0]) + np.outer(A1[0], A0[1]) + np.outer(A1[1], A0[1])
    out[:, 1] += np.einsum("ekji,k,ji->e", f, A2[1], top)
    return out


def iproduct(yb, jac, phys):
    phys = np.asarray(phys, dtype=np.float64).reshape(-1, yb.nq)
    E = phys.shape[0]
    return iproduct_tables(yb, yb.B0, yb.B0, yb.B2, phys * _pts(jac, E, yb.nq) * yb.weights()[None])


def collapsed_derivs(yb, phys):
    u = np.asarray(phys, dtype=np.float64).reshape(-1, yb.Q2, yb.Q1, yb.Q0)
    E = u.shape[0]
    d0 = np.einsum("ab,ekjb->ekja", yb.D0_2, u)
    d1 = np.einsum("ab,ekbi->ekai", yb.D0_2, u)
    d2 = np.einsum("ab,ebji->eaji", yb.D2_2, u)
    return [d.reshape(E, -1) for d in (d0, d1, d2)]


def _factors(yb):
    """Per point: h0 = (1+z0_i)/2, h1 = (1+z0_j)/2, h2 = 2/(1-z2_k)."""
    Q0 = yb.Q0
    H0 = np.tile(0.5 * (1 + yb.z0), Q0 * yb.Q2)[None]
    H1 = np.tile(np.repeat(0.5 * (1 + yb.z0), Q0), yb.Q2)[None]
    H2 = np.repeat(2.0 / (1 - yb.z2), Q0 * Q0)[None]
    return H0, H1, H2


def xi_derivs(yb, phys):
    d0, d1, d2 = collapsed_derivs(yb, phys)
    H0, H1, H2 = _factors(yb)
    x0, x1 = H2 * d0, H2 * d1
    return x0, x1, H0 * x0 + H1 * x1 + d2


def physderiv(yb, df, phys):
    u = np.asarray(phys, dtype=np.float64).reshape(-1, yb.nq)
    E = u.shape[0]
    x = xi_derivs(yb, u)
    f = [_pts(df[k], E, yb.nq) for k in range(9)]
    return [sum(f[c * 3 + j] * x[j] for j in range(3)) for c in range(3)]


def helmholtz(yb, jac, df, lam, coeffs):
    """lambda M u + L u, composed as HelmholtzPyrImpl."""
    c = np.asarray(coeffs, dtype=np.float64).reshape(-1, yb.nc)
    E = c.shape[0]
    nq = yb.nq
    J = _pts(jac, E, nq)
    W = yb.weights()[None]
    bwd = bwdtrans(yb, c)
    out = lam * iproduct_tables(yb, yb.B0, yb.B0, yb.B2, bwd * J * W)
    d0, d1, d2 = collapsed_derivs(yb, bwd)
    H0, H1, H2 = _factors(yb)
    f = [_pts(df[k], E, nq) for k in range(9)]
    a = [H2 * (f[3 * cc] + H0 * f[3 * cc + 2]) for cc in range(3)]
    b = [H2 * (f[3 * cc + 1] + H1 * f[3 * cc + 2]) for cc in range(3)]
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
    out = out + iproduct_tables(yb, yb.DB0, yb.B0, yb.B2, t0 * J * W)
    out = out + iproduct_tables(yb, yb.B0, yb.DB0, yb.B2, t1 * J * W)
    out = out + iproduct_tables(yb, yb.B0, yb.B0, yb.DB2, t2 * J * W)
    return out


def iproduct_deriv(yb, jac, df, comps):
    cs = [np.asarray(x, dtype=np.float64).reshape(-1, yb.nq) for x in comps]
    E = cs[0].shape[0]
    J = _pts(jac, E, yb.nq)
    W = yb.weights()[None]
    f = [_pts(df[k], E, yb.nq) for k in range(9)]
    t = [sum(f[3 * c + j] * cs[c] for c in range(3)) for j in range(3)]
    H0, H1, H2 = _factors(yb)
    return (iproduct_tables(yb, yb.DB0, yb.B0, yb.B2, H2 * (t[0] + H0 * t[2]) * J * W) +
            iproduct_tables(yb, yb.B0, yb.DB0, yb.B2, H2 * (t[1] + H1 * t[2]) * J * W) +
            iproduct_tables(yb, yb.B0, yb.B0, yb.DB2, t[2] * J * W))


def helmholtz_diag(yb, E, jac, df, lam):
    d = np.zeros((E, yb.nc))
    for m in range(yb.nc):
        u = np.zeros((E, yb.nc))
        u[:, m] = 1.0
        d[:, m] = helmholtz(yb, jac, df, lam, u)[:, m]
    return d


def geom_factors(yb, X):
    X = np.asarray(X, dtype=np.float64)
    E = X.shape[1]
    dx = np.stack([np.stack(xi_derivs(yb, X[c])) for c in range(3)])
    M = np.moveaxis(dx, (0, 1), (-2, -1))
    J = np.linalg.det(M)
    inv = np.linalg.inv(M)
    df = np.stack([inv[..., j, c] for c in range(3) for j in range(3)]).reshape(9, E * yb.nq)
    return J, df


def modal_values(n, xi0, xi1, xi2):
    """phi_m at reference points with xi2 < 1: (npts, nc); mode 1 (the apex) is (1 + eta2)/2."""
    xi0, xi1, xi2 = (np.asarray(a, dtype=np.float64) for a in (xi0, xi1, xi2))
    e0 = 2 * (1 + xi0) / (1 - xi2) - 1
    e1 = 2 * (1 + xi1) / (1 - xi2) - 1
    shape = np.broadcast(e0, e1, xi2).shape

    def modA(p, x):
        if p == 0:
            return 0.5 * (1 - x)
        if p == 1:
            return 0.5 * (1 + x)
        return 0.25 * (1 - x) * (1 + x) * polylib.jacobi(p - 2, 1.0, 1.0, x)
    C = pyrC_rows(n, np.broadcast_to(xi2, shape).reshape(-1)).reshape((-1,) + shape)
    cols = []
    for m, (p, q, r) in enumerate(pyr_modes(n)):
        if m == 1:
            cols.append(0.5 * (1 + np.broadcast_to(xi2, shape)))
        else:
            cols.append(modA(p, e0) * modA(q, e1) * C[m])
    return np.stack(cols, axis=-1)
