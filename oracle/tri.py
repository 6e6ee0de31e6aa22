"""Triangle element operators (oracle restatement, FP64). Test infrastructure only.

Expansion (the default keys of SpatialDomains/MeshGraph.cpp:1665-1681):
  direction 0  eModified_A, n modes on Q0 = n + 1 Gauss-Lobatto-Legendre points
  direction 1  eModified_B, n (n + 1) / 2 modes on Q1 = n Gauss-Radau-Jacobi points
               (alpha 1, beta 0; z = -1 included), LibUtilities/Foundations/Basis.cpp:423-507
Mode index m(p, q) runs q fastest over 0 <= p < n, 0 <= q < n - p. Physical layout
u[e, j*Q0 + i] (i along the collapsed coordinate eta0). Geometry as for quads: ``jac``
(E,) or (E, Q0*Q1), ``df`` (4, E) or (4, E*Q0*Q1) with df[k*2 + j] = d xi_j / d x_k.

Operators restate the MatrixFree triangle kernels, CORRECT = true (eModified_A):
  bwdtrans   MatrixFreeOps/BwdTransKernels.hpp:78-125  (BwdTransTriKernel)
  iproduct   MatrixFreeOps/IProductKernels.hpp:136-234 (IProductTriKernel): the
             Gauss-Radau weights carry the factor 0.5 of MatrixFreeOps/Operator.hpp:245-248
  physderiv  MatrixFreeOps/PhysDerivKernels.hpp:153-212 (PhysDerivTriKernel)
  helmholtz  MatrixFreeOps/Helmholtz.h:290-330, 505-635 (HelmholtzTriImpl)
The singular vertex: mode m = 1 (p = 0, q = 1) is the top vertex; the kernels add
c_1 B0_1(eta0) B1_1(eta1) in BwdTrans and the matching term to out[1] in IProduct, which
makes the vertex function (1 + eta1)/2 over the whole element.

Quadrature rules are computed by a different route from Polylib (zwgrjm / Dgrjm):
the Radau interior points are the eigenvalues of the Jacobi matrix of P^{(1,1)}
(Golub-Welsch) polished by Newton, the weights solve the Legendre moment equations of
the weight (1 - z), and D is the barycentric Lagrange derivative.
"""
import numpy as np

from . import polylib
from .basis import Basis1D


def _jacobi_deriv(n, a, b, z):
    """d/dz P_n^{(a,b)} = (n + a + b + 1)/2 P_{n-1}^{(a+1,b+1)}."""
    if n == 0:
        return np.zeros_like(np.asarray(z, dtype=np.float64))
    return 0.5 * (n + a + b + 1.0) * polylib.jacobi(n - 1, a + 1.0, b + 1.0, z)


def _jacobi_zeros(n, a, b):
    """Zeros of P_n^{(a,b)}: Golub-Welsch eigenvalues, then Newton on the recurrence."""
    if n == 0:
        return np.zeros(0)
    k = np.arange(n, dtype=np.float64)
    apb = a + b
    diag = np.where(2 * k + apb == 0, (b - a) / (apb + 2.0),
                    (b * b - a * a) / np.maximum((2 * k + apb) * (2 * k + apb + 2.0), 1e-300))
    kk = np.arange(1, n, dtype=np.float64)
    off = 2.0 / (2 * kk + apb) * np.sqrt(kk * (kk + a) * (kk + b) * (kk + apb) /
                                         ((2 * kk + apb - 1.0) * (2 * kk + apb + 1.0)))
    J = np.diag(diag) + np.diag(off, 1) + np.diag(off, -1)
    z = np.sort(np.linalg.eigvalsh(J))
    for _ in range(50):
        step = polylib.jacobi(n, a, b, z) / _jacobi_deriv(n, a, b, z)
        z = z - step
        if np.max(np.abs(step)) < 1e-16:
            break
    return z


def radau_m(Q):
    """Gauss-Radau-Jacobi points (z_0 = -1) and weights for the weight (1 - z)."""
    if Q == 1:
        return np.zeros(1), np.full(1, 2.0)
    z = np.concatenate([[-1.0], _jacobi_zeros(Q - 1, 1.0, 1.0)])
    # sum_i w_i P_k(z_i) = int_{-1}^{1} (1 - z) P_k(z) dz = 2 [k = 0] - 2/3 [k = 1]
    V = np.stack([polylib.jacobi(k, 0.0, 0.0, z) for k in range(Q)])
    mom = np.zeros(Q)
    mom[0] = 2.0
    if Q > 1:
        mom[1] = -2.0 / 3.0
    w = np.linalg.solve(V, mom)
    return z, w


def lagrange_d(z):
    """Flattened collocation derivative, D[k*Q + i] = l_k'(z_i) (barycentric form)."""
    Q = len(z)
    diff = z[:, None] - z[None, :]
    np.fill_diagonal(diff, 1.0)
    c = np.prod(diff, axis=1)  # c_i = prod_{j != i} (z_i - z_j)
    D2 = np.zeros((Q, Q))      # D2[i, k] = l_k'(z_i)
    for i in range(Q):
        for k in range(Q):
            if i != k:
                D2[i, k] = c[i] / (c[k] * (z[i] - z[k]))
        D2[i, i] = np.sum(1.0 / (z[i] - np.delete(z, i)))
    return D2.T.reshape(-1).copy()


def mode_rows(n):
    """p of each triangular mode index m(p, q), q fastest."""
    return np.concatenate([np.full(n - p, p) for p in range(n)])


class TriBasis:
    """Tables of one triangle expansion with n modes per direction."""

    def __init__(self, n):
        self.n = n
        self.Q0, self.Q1 = n + 1, n
        self.nc = n * (n + 1) // 2
        a = Basis1D(n, n + 1)
        self.z0, self.w0, self.D0 = a.z, a.w, a.D
        self.B0, self.DB0 = a.B2, a.DB2          # [p, i]
        self.D0_2 = a.D2                          # [i, k] = l_k'(z_i)
        Q1 = self.Q1
        self.z1, self.w1 = radau_m(Q1)
        self.D1 = lagrange_d(self.z1)
        self.D1_2 = self.D1.reshape(Q1, Q1).T
        z = self.z1
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
        self.B1 = np.array(rows)                  # [m, j]
        self.DB1 = (self.D1_2 @ self.B1.T).T      # DB1[m, j] = sum_l D1(j, l) B1[m, l]
        self.w1h = 0.5 * self.w1                  # the MatrixFree Helper's weight factor
        self.h0 = 0.5 * (1.0 + self.z0)
        self.h1 = 2.0 / (1.0 - self.z1)
        self.prow = mode_rows(n)
        self.Prow = np.zeros((n, self.nc))        # Prow[p, m] = 1 if mode m is in row p
        self.Prow[self.prow, np.arange(self.nc)] = 1.0

    @property
    def nq(self):
        return self.Q0 * self.Q1


def _pts(a, E, nq):
    a = np.asarray(a, dtype=np.float64)
    if a.size == E:
        return np.repeat(a.reshape(E, 1), nq, axis=1)
    return a.reshape(E, nq)


def bwdtrans(tb, coeffs):
    c = np.asarray(coeffs, dtype=np.float64).reshape(-1, tb.nc)
    E = c.shape[0]
    ps = np.einsum("pm,mj,em->epj", tb.Prow, tb.B1, c)
    ps[:, 1, :] += c[:, 1:2] * tb.B1[1][None, :]   # singular vertex
    u = np.einsum("epj,pi->eji", ps, tb.B0)
    return u.reshape(E, tb.nq)


def iproduct_tables(tb, A0, A1, fw):
    """out[m] = sum_ij A0[p(m), i] A1[m, j] fw[j, i] + the singular-vertex term to m = 1;
    fw is the field already multiplied by J w0 w1h."""
    E = fw.shape[0]
    f = fw.reshape(E, tb.Q1, tb.Q0)
    g = np.einsum("pi,eji->epj", A0, f)
    out = np.einsum("mj,emj->em", A1, g[:, tb.prow, :])
    out[:, 1] += g[:, 1, :] @ A1[1]
    return out


def _weights(tb):
    return np.outer(tb.w1h, tb.w0).reshape(-1)


def iproduct(tb, jac, phys):
    phys = np.asarray(phys, dtype=np.float64).reshape(-1, tb.nq)
    E = phys.shape[0]
    J = _pts(jac, E, tb.nq)
    return iproduct_tables(tb, tb.B0, tb.B1, phys * J * _weights(tb)[None])


def collapsed_derivs(tb, phys):
    u = np.asarray(phys, dtype=np.float64).reshape(-1, tb.Q1, tb.Q0)
    E = u.shape[0]
    d0 = np.einsum("ab,ejb->eja", tb.D0_2, u)
    d1 = np.einsum("ab,ebi->eai", tb.D1_2, u)
    return d0.reshape(E, -1), d1.reshape(E, -1)


def physderiv(tb, df, phys):
    u = np.asarray(phys, dtype=np.float64).reshape(-1, tb.nq)
    E = u.shape[0]
    d0, d1 = collapsed_derivs(tb, u)
    H0 = np.tile(tb.h0, tb.Q1)[None]
    H1 = np.repeat(tb.h1, tb.Q0)[None]
    x0 = H1 * d0                 # d/dxi0
    x1 = d1 + H0 * x0            # d/dxi1
    f = [_pts(df[k], E, tb.nq) for k in range(4)]
    return f[0] * x0 + f[1] * x1, f[2] * x0 + f[3] * x1


def helmholtz(tb, jac, df, lam, coeffs, kappa=None):
    """lambda M u + L u, composed as HelmholtzTriImpl; kappa (E, nq) scales the Laplacian
    per point (an isotropic variable coefficient, StdExpansion.cpp:664-717)."""
    c = np.asarray(coeffs, dtype=np.float64).reshape(-1, tb.nc)
    E = c.shape[0]
    nq = tb.nq
    J = _pts(jac, E, nq)
    W = _weights(tb)[None]
    bwd = bwdtrans(tb, c)
    out = lam * iproduct_tables(tb, tb.B0, tb.B1, bwd * J * W)
    d0, d1 = collapsed_derivs(tb, bwd)
    f = [_pts(df[k], E, nq) for k in range(4)]
    H0 = np.tile(tb.h0, tb.Q1)[None]
    H1 = np.repeat(tb.h1, tb.Q0)[None]
    a = H1 * (f[0] + H0 * f[1])
    b = H1 * (f[2] + H0 * f[3])
    m00 = a * a + b * b
    m01 = a * f[1] + b * f[3]
    m11 = f[1] * f[1] + f[3] * f[3]
    t0 = m00 * d0 + m01 * d1
    t1 = m01 * d0 + m11 * d1
    if kappa is not None:
        k = np.asarray(kappa, dtype=np.float64).reshape(E, nq)
        t0, t1 = k * t0, k * t1
    out = out + iproduct_tables(tb, tb.DB0, tb.B1, t0 * J * W)
    out = out + iproduct_tables(tb, tb.B0, tb.DB1, t1 * J * W)
    return out


def iproduct_deriv(tb, jac, df, comps):
    """sum_k (d phi / d x_k, comps[k]) (IProductWRTDerivBaseTriImpl, MatrixFreeOps/
    IProductWRTDerivBase.h:671-1060): t_j = sum_k df[k*2+j] comps[k]; the xi derivatives
    of phi in collapsed form give IProduct_{DB0,B1}(h1 (t_0 + h0 t_1)) + IProduct_{B0,DB1}(t_1)."""
    c0 = np.asarray(comps[0], dtype=np.float64).reshape(-1, tb.nq)
    c1 = np.asarray(comps[1], dtype=np.float64).reshape(-1, tb.nq)
    E = c0.shape[0]
    J = _pts(jac, E, tb.nq)
    W = _weights(tb)[None]
    f = [_pts(df[k], E, tb.nq) for k in range(4)]
    t0 = f[0] * c0 + f[2] * c1
    t1 = f[1] * c0 + f[3] * c1
    H0 = np.tile(tb.h0, tb.Q1)[None]
    H1 = np.repeat(tb.h1, tb.Q0)[None]
    a = H1 * (t0 + H0 * t1)
    return (iproduct_tables(tb, tb.DB0, tb.B1, a * J * W) +
            iproduct_tables(tb, tb.B0, tb.DB1, t1 * J * W))


def helmholtz_diag(tb, E, jac, df, lam):
    """Diagonal of every element's Helmholtz matrix (one apply per mode), (E, nc)."""
    d = np.zeros((E, tb.nc))
    for m in range(tb.nc):
        u = np.zeros((E, tb.nc))
        u[:, m] = 1.0
        d[:, m] = helmholtz(tb, jac, df, lam, u)[:, m]
    return d


def modal_values(n, eta0, eta1):
    """phi_m at arbitrary collapsed points (arrays eta0, eta1): (npts, nc), the top vertex
    m = 1 with the singular-vertex term, i.e. (1 + eta1)/2."""
    eta0 = np.asarray(eta0, dtype=np.float64)
    eta1 = np.asarray(eta1, dtype=np.float64)
    a0, a1 = 0.5 * (1.0 - eta0), 0.5 * (1.0 + eta0)
    lo, hi = 0.5 * (1.0 - eta1), 0.5 * (1.0 + eta1)
    cols = []
    for p in range(n):
        A = a0 if p == 0 else (a1 if p == 1 else a0 * a1 * polylib.jacobi(p - 2, 1.0, 1.0, eta0))
        for q in range(n - p):
            if p == 0:
                Bv = lo if q == 0 else (hi if q == 1 else lo * hi * polylib.jacobi(q - 2, 1.0, 1.0, eta1))
            elif q == 0:
                Bv = lo ** p
            else:
                Bv = lo ** p * hi * polylib.jacobi(q - 1, 2.0 * p - 1.0, 1.0, eta1)
            cols.append(A * Bv)
    V = np.stack(cols, axis=-1)
    V[..., 1] = hi
    return V


def geom_factors(tb, X):
    """Jacobian and derivative factors at the quadrature points of triangles whose
    coordinates X (2, E, Q0*Q1) are given there: the collapsed derivatives mapped to
    d/dxi0 = h1 d/deta0, d/dxi1 = h0 h1 d/deta0 + d/deta1 (the chain rule of
    StdTriExp::v_PhysDeriv), then J = det and df = the inverse of dx/dxi."""
    X = np.asarray(X, dtype=np.float64)
    E = X.shape[1]
    H0 = np.tile(tb.h0, tb.Q1)[None]
    H1 = np.repeat(tb.h1, tb.Q0)[None]
    dx = []
    for c in range(2):
        d0, d1 = collapsed_derivs(tb, X[c])
        x0 = H1 * d0
        dx.append((x0, d1 + H0 * x0))   # (dx_c/dxi0, dx_c/dxi1)
    (xa, xb), (ya, yb) = dx
    J = xa * yb - xb * ya
    df = np.stack([yb / J, -ya / J, -xb / J, xa / J]).reshape(4, E * tb.nq)
    return J, df


def straight_tri_geometry(V):
    """Per-element (regular) J and df of straight-sided triangles with vertices V (E, 3, 2):
    x = v0 + (v1 - v0)(1 + xi0)/2 + (v2 - v0)(1 + xi1)/2."""
    V = np.asarray(V, dtype=np.float64)
    a = 0.5 * (V[:, 1] - V[:, 0])
    b = 0.5 * (V[:, 2] - V[:, 0])
    J = a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]
    df = np.stack([b[:, 1] / J, -a[:, 1] / J, -b[:, 0] / J, a[:, 0] / J])
    return J, df
