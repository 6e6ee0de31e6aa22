"""Tetrahedron element operators (oracle restatement, FP64). Test infrastructure only.

Expansion (the default keys of SpatialDomains/MeshGraph.cpp:1683-1716):
  direction 0  eModified_A, n modes on Q0 = n + 1 Gauss-Lobatto-Legendre points
  direction 1  eModified_B on Q1 = n Gauss-Radau-Jacobi points (alpha 1, beta 0)
  direction 2  eModified_C on Q2 = n Gauss-Radau-Jacobi points (alpha 2, beta 0);
               phi^c_{pqr} = phi^b_{p+q,r} (LibUtilities/Foundations/Basis.cpp:512-566)
Modes m(p, q, r): r fastest, then q, then p, 0 <= p < n, q < n - p, r < n - p - q
(n (n+1) (n+2) / 6 of them). Physical layout u[e, (k Q1 + j) Q0 + i]. Geometry: ``jac``
(E,) or (E, nq); ``df`` (9, E) or (9, E nq) with df[c*3 + j] = d xi_j / d x_c.

Operators restate the MatrixFree tetrahedron kernels with CORRECT = true:
  bwdtrans   MatrixFreeOps/BwdTransKernels.hpp:374-480 (BwdTransTetKernel): the top vertex
             (mode 1), the bottom vertex (mode n) and the singular edge (modes n + r)
  iproduct   MatrixFreeOps/IProductKernels.hpp:601-790 (IProductTetKernel), Gauss-Radau
             weights times 0.5 (alpha 1) and 0.25 (alpha 2), MatrixFreeOps/Operator.hpp:245-251
  physderiv  MatrixFreeOps/PhysDerivKernels.hpp:555-700 (PhysDerivTetKernel)
  helmholtz  MatrixFreeOps/Helmholtz.h:1970-2010, 2266-2448 (HelmholtzTetImpl)
  iproduct_deriv  MatrixFreeOps/IProductWRTDerivBase.h:2212-2630
The quadrature rules come from oracle/tri.py's route (Golub-Welsch points, Legendre
moments for the weights, barycentric D), not from Polylib.
"""
import numpy as np

from . import polylib
from .basis import Basis1D
from .tri import _jacobi_zeros, lagrange_d


def radau_m(Q, alpha):
    """Gauss-Radau-Jacobi points (z_0 = -1) and weights for the weight (1 - z)^alpha."""
    if Q == 1:
        return np.zeros(1), np.full(1, 2.0)
    z = np.concatenate([[-1.0], _jacobi_zeros(Q - 1, float(alpha), 1.0)])
    g, wg = np.polynomial.legendre.leggauss(Q + 4)
    V = np.stack([polylib.jacobi(k, 0.0, 0.0, z) for k in range(Q)])
    mom = np.array([np.sum(wg * (1.0 - g) ** alpha * polylib.jacobi(k, 0.0, 0.0, g)) for k in range(Q)])
    return z, np.linalg.solve(V, mom)


def modB_rows(n, z):
    """eModified_B rows (p, q), q fastest (Basis.cpp:423-507)."""
    lo, hi = 0.5 * (1.0 - z), 0.5 * (1.0 + z)
    rows = []
    for p in range(n):
        for q in range(n - p):
            if p == 0:
                r = lo if q == 0 else (hi if q == 1 else lo * hi * polylib.jacobi(q - 2, 1.0, 1.0, z))
            elif q == 0:
                r = lo ** p
            else:
                r = lo ** p * hi * polylib.jacobi(q - 1, 2.0 * p - 1.0, 1.0, z)
            rows.append(r)
    return np.array(rows)


def tet_modes(n):
    return [(p, q, r) for p in range(n) for q in range(n - p) for r in range(n - p - q)]


def pair_index(n, p, q):
    return sum(n - pp for pp in range(p)) + q


class TetBasis:
    def __init__(self, n):
        self.n = n
        self.Q0, self.Q1, self.Q2 = n + 1, n, n
        a = Basis1D(n, n + 1)
        self.z0, self.w0, self.D0 = a.z, a.w, a.D
        self.B0, self.DB0, self.D0_2 = a.B2, a.DB2, a.D2
        self.z1, self.w1 = radau_m(n, 1)
        self.z2, self.w2 = radau_m(n, 2)
        self.D1, self.D2 = lagrange_d(self.z1), lagrange_d(self.z2)
        self.D1_2 = self.D1.reshape(n, n).T
        self.D2_2 = self.D2.reshape(n, n).T
        self.B1 = modB_rows(n, self.z1)                       # [pq, j]
        self.DB1 = (self.D1_2 @ self.B1.T).T
        modes = tet_modes(n)
        self.modes = modes
        self.nc = len(modes)
        b2 = modB_rows(n, self.z2)
        self.B2 = np.array([b2[pair_index(n, p + q, r)] for (p, q, r) in modes])   # [m, k]
        self.DB2 = (self.D2_2 @ self.B2.T).T
        self.w1h, self.w2h = 0.5 * self.w1, 0.25 * self.w2
        self.npq = n * (n + 1) // 2
        self.pq_of = np.array([pair_index(n, p, q) for (p, q, r) in modes])
        self.p_of_pq = np.concatenate([np.full(n - p, p) for p in range(n)])
        self.nq = self.Q0 * self.Q1 * self.Q2

    def weights(self):
        return (self.w2h[:, None, None] * self.w1h[None, :, None] * self.w0[None, None, :]).reshape(-1)


def _pts(a, E, nq):
    a = np.asarray(a, dtype=np.float64)
    if a.size == E:
        return np.repeat(a.reshape(E, 1), nq, axis=1)
    return a.reshape(E, nq)


def bwdtrans(tb, coeffs):
    n = tb.n
    c = np.asarray(coeffs, dtype=np.float64).reshape(-1, tb.nc)
    E = c.shape[0]
    F = np.zeros((E, tb.npq, tb.Q2))
    np.add.at(F, (slice(None), tb.pq_of), c[:, :, None] * tb.B2[None])
    G = np.zeros((E, n, tb.Q1, tb.Q2))
    for pq in range(tb.npq):
        G[:, tb.p_of_pq[pq]] += tb.B1[pq][None, :, None] * F[:, pq][:, None, :]
    u = np.einsum("pi,epjk->ekji", tb.B0, G)
    # singular-vertex and singular-edge terms, written as BwdTransTetKernel adds them
    B0, B1, B2 = tb.B0, tb.B1, tb.B2
    top = (np.outer(B1[1], B0[0]) + np.outer(B1[0], B0[1]) + np.outer(B1[1], B0[1]))   # [j, i]
    u += c[:, 1][:, None, None, None] * B2[1][None, :, None, None] * top[None, None]
    e11 = np.outer(B1[1], B0[1])
    u += c[:, n][:, None, None, None] * B2[0][None, :, None, None] * e11[None, None]
    for r in range(1, n - 1):
        u += c[:, n + r][:, None, None, None] * B2[r + 1][None, :, None, None] * e11[None, None]
    return u.reshape(E, tb.nq)


def iproduct_tables(tb, A0, A1, A2, fw):
    """IProductTetKernel with tables A0 (p), A1 (pq), A2 (m) on a field fw already
    multiplied by J w; the CORRECT terms to modes 1, n and n + r."""
    n = tb.n
    E = fw.shape[0]
    f = fw.reshape(E, tb.Q2, tb.Q1, tb.Q0)
    G = np.einsum("pi,ekji->epjk", A0, f)
    F = np.einsum("Pj,ePjk->ePk", A1, G[:, tb.p_of_pq])
    out = np.einsum("mk,emk->em", A2, F[:, tb.pq_of])
    top = (np.outer(A1[1], A0[0]) + np.outer(A1[0], A0[1]) + np.outer(A1[1], A0[1]))
    out[:, 1] += np.einsum("ekji,k,ji->e", f, A2[1], top)
    e11 = np.outer(A1[1], A0[1])
    out[:, n] += np.einsum("ekji,k,ji->e", f, A2[0], e11)
    for r in range(1, n - 1):
        out[:, n + r] += np.einsum("ekji,k,ji->e", f, A2[r + 1], e11)
    return out


def iproduct(tb, jac, phys):
    phys = np.asarray(phys, dtype=np.float64).reshape(-1, tb.nq)
    E = phys.shape[0]
    J = _pts(jac, E, tb.nq)
    return iproduct_tables(tb, tb.B0, tb.B1, tb.B2, phys * J * tb.weights()[None])


def collapsed_derivs(tb, phys):
    u = np.asarray(phys, dtype=np.float64).reshape(-1, tb.Q2, tb.Q1, tb.Q0)
    E = u.shape[0]
    d0 = np.einsum("ab,ekjb->ekja", tb.D0_2, u)
    d1 = np.einsum("ab,ekbi->ekai", tb.D1_2, u)
    d2 = np.einsum("ab,ebji->eaji", tb.D2_2, u)
    return [d.reshape(E, -1) for d in (d0, d1, d2)]


def _factors(tb):
    """Per point: h0 = (1+z0)/2, h1 = (1+z1)/2, h2 = 2/(1-z1), h3 = 2/(1-z2)."""
    Q0, Q1, Q2 = tb.Q0, tb.Q1, tb.Q2
    H0 = np.tile(0.5 * (1 + tb.z0), Q1 * Q2)[None]
    H1 = np.tile(np.repeat(0.5 * (1 + tb.z1), Q0), Q2)[None]
    H2 = np.tile(np.repeat(2.0 / (1 - tb.z1), Q0), Q2)[None]
    H3 = np.repeat(2.0 / (1 - tb.z2), Q0 * Q1)[None]
    return H0, H1, H2, H3


def xi_derivs(tb, phys):
    d0, d1, d2 = collapsed_derivs(tb, phys)
    H0, H1, H2, H3 = _factors(tb)
    x0 = H2 * H3 * d0
    x1 = H0 * x0 + H3 * d1
    x2 = H0 * x0 + H1 * H3 * d1 + d2
    return x0, x1, x2


def physderiv(tb, df, phys):
    u = np.asarray(phys, dtype=np.float64).reshape(-1, tb.nq)
    E = u.shape[0]
    x = xi_derivs(tb, u)
    f = [_pts(df[k], E, tb.nq) for k in range(9)]
    return [sum(f[c * 3 + j] * x[j] for j in range(3)) for c in range(3)]


def helmholtz(tb, jac, df, lam, coeffs):
    """lambda M u + L u, composed as HelmholtzTetImpl."""
    c = np.asarray(coeffs, dtype=np.float64).reshape(-1, tb.nc)
    E = c.shape[0]
    nq = tb.nq
    J = _pts(jac, E, nq)
    W = tb.weights()[None]
    bwd = bwdtrans(tb, c)
    out = lam * iproduct_tables(tb, tb.B0, tb.B1, tb.B2, bwd * J * W)
    d0, d1, d2 = collapsed_derivs(tb, bwd)
    H0, H1, H2, H3 = _factors(tb)
    f = [_pts(df[k], E, nq) for k in range(9)]
    a = [H2 * H3 * f[3 * cc] + H0 * H2 * H3 * (f[3 * cc + 1] + f[3 * cc + 2]) for cc in range(3)]
    b = [H3 * f[3 * cc + 1] + H1 * H3 * f[3 * cc + 2] for cc in range(3)]
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
    out = out + iproduct_tables(tb, tb.DB0, tb.B1, tb.B2, t0 * J * W)
    out = out + iproduct_tables(tb, tb.B0, tb.DB1, tb.B2, t1 * J * W)
    out = out + iproduct_tables(tb, tb.B0, tb.B1, tb.DB2, t2 * J * W)
    return out


def iproduct_deriv(tb, jac, df, comps):
    """sum_c (d phi / d x_c, comps[c]) (IProductWRTDerivBaseTetImpl)."""
    cs = [np.asarray(x, dtype=np.float64).reshape(-1, tb.nq) for x in comps]
    E = cs[0].shape[0]
    J = _pts(jac, E, tb.nq)
    W = tb.weights()[None]
    f = [_pts(df[k], E, tb.nq) for k in range(9)]
    t = [sum(f[3 * c + j] * cs[c] for c in range(3)) for j in range(3)]
    H0, H1, H2, H3 = _factors(tb)
    a = H2 * H3 * (t[0] + H0 * (t[1] + t[2]))
    b = H3 * (t[1] + H1 * t[2])
    return (iproduct_tables(tb, tb.DB0, tb.B1, tb.B2, a * J * W) +
            iproduct_tables(tb, tb.B0, tb.DB1, tb.B2, b * J * W) +
            iproduct_tables(tb, tb.B0, tb.B1, tb.DB2, t[2] * J * W))


def helmholtz_diag(tb, E, jac, df, lam):
    d = np.zeros((E, tb.nc))
    for m in range(tb.nc):
        u = np.zeros((E, tb.nc))
        u[:, m] = 1.0
        d[:, m] = helmholtz(tb, jac, df, lam, u)[:, m]
    return d


def collapsed_to_xi(z0, z1, z2):
    """(xi0, xi1, xi2) at the collapsed points, arrays [k, j, i]."""
    e2, e1, e0 = np.meshgrid(z2, z1, z0, indexing="ij")
    xi2 = e2
    xi1 = 0.5 * (1 + e1) * (1 - e2) - 1
    xi0 = 0.25 * (1 + e0) * (1 - e1) * (1 - e2) - 1
    return xi0, xi1, xi2


def geom_factors(tb, X):
    """J and df at the collapsed points from coordinates X (3, E, nq) there."""
    X = np.asarray(X, dtype=np.float64)
    E = X.shape[1]
    dx = np.stack([np.stack(xi_derivs(tb, X[c])) for c in range(3)])   # [c, j, E, nq] = dx_c/dxi_j
    M = np.moveaxis(dx, (0, 1), (-2, -1))                              # [E, nq, c, j]
    J = np.linalg.det(M)
    inv = np.linalg.inv(M)                                             # [E, nq, j, c] = dxi_j/dx_c
    df = np.stack([inv[..., j, c] for c in range(3) for j in range(3)]).reshape(9, E * tb.nq)
    return J, df


def straight_tet_geometry(V):
    """Per-element J and df of straight tetrahedra (E, 4, 3):
    x = v0 + (v1-v0)(1+xi0)/2 + (v2-v0)(1+xi1)/2 + (v3-v0)(1+xi2)/2."""
    V = np.asarray(V, dtype=np.float64)
    M = 0.5 * np.stack([V[:, 1] - V[:, 0], V[:, 2] - V[:, 0], V[:, 3] - V[:, 0]], axis=2)  # [E, c, j]
    J = np.linalg.det(M)
    inv = np.linalg.inv(M)
    df = np.stack([inv[:, j, c] for c in range(3) for j in range(3)])
    return J, df


def modal_values(n, xi0, xi1, xi2):
    """phi_m at reference points away from the collapsed edge (xi1 + xi2 < 0, xi2 < 1):
    (npts, nc); the top vertex (0,0,1) is (1 + eta2)/2 and the modes (0,1,r) carry no eta0
    factor (the CORRECT terms of BwdTransTetKernel)."""
    xi0, xi1, xi2 = (np.asarray(a, dtype=np.float64) for a in (xi0, xi1, xi2))
    e2 = xi2
    e1 = 2 * (1 + xi1) / (1 - xi2) - 1
    e0 = 2 * (1 + xi0) / (-xi1 - xi2) - 1
    shape = np.broadcast(e0, e1, e2).shape
    A = [polylib_modA(p, e0) for p in range(n)]
    B1 = modB_rows(n, e1.reshape(-1)).reshape((-1,) + shape)
    B2 = modB_rows(n, e2.reshape(-1)).reshape((-1,) + shape)
    cols = []
    for (p, q, r) in tet_modes(n):
        if (p, q, r) == (0, 0, 1):
            cols.append(0.5 * (1 + e2) * np.ones(shape))
            continue
        x = np.ones(shape) if (p == 0 and q == 1) else A[p]
        cols.append(x * B1[pair_index(n, p, q)] * B2[pair_index(n, p + q, r)])
    return np.stack(cols, axis=-1)


def polylib_modA(p, x):
    if p == 0:
        return 0.5 * (1 - x)
    if p == 1:
        return 0.5 * (1 + x)
    return 0.25 * (1 - x) * (1 + x) * polylib.jacobi(p - 2, 1.0, 1.0, x)
