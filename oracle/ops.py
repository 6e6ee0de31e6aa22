"""Element operators on quads and hexes (oracle restatement, FP64).

Layouts are the reference's element-contiguous ones:
  coefficients  quad  u[e, q*n + p]              hex  u[e, (r*n + q)*n + p]
  physical      quad  u[e, j*Q + i]              hex  u[e, (k*Q + j)*Q + i]
(p / i run along direction 0 and are fastest). Geometry: ``jac`` is (E, Q^d) for
deformed collections or (E,) for regular ones; ``df`` is (d*d, E*Q^d) or (d*d, E).

Each function restates the composition of the reference MatrixFree kernels:
  bwdtrans   MatrixFreeOps/BwdTransKernels.hpp:35-76 (quad), :302-372 (hex)
  iproduct   MatrixFreeOps/IProductKernels.hpp:76-133 (quad), :236-314 (hex)
  physderiv  MatrixFreeOps/PhysDerivKernels.hpp:39-151 (quad), :219-374 (hex)
  helmholtz  MatrixFreeOps/Helmholtz.h:137-275 (quad), :763-993 (hex)
  iproduct_deriv  Collections/IProductWRTDerivBase.cpp:446-546 (IterPerExp)
with einsum in place of the SIMD loops (same sums, different summation order).
"""
import numpy as np


def _geo_pts(a, E, nq):
    """Broadcast per-element (regular) or per-point (deformed) data to (E, nq)."""
    a = np.asarray(a)
    if a.size == E:
        return np.repeat(a.reshape(E, 1), nq, axis=1)
    return a.reshape(E, nq)


def _df_pts(df, dim, E, nq):
    return [_geo_pts(df[k], E, nq) for k in range(dim * dim)]


def bwdtrans(basis, dim, coeffs):
    b = basis
    n, Q = b.n, b.Q
    E = coeffs.size // n ** dim
    if dim == 2:
        c = coeffs.reshape(E, n, n)  # [e, q, p]
        return np.einsum('qj,pi,eqp->eji', b.B2, b.B2, c, optimize=True).reshape(E, -1)
    c = coeffs.reshape(E, n, n, n)   # [e, r, q, p]
    return np.einsum('rk,qj,pi,erqp->ekji', b.B2, b.B2, b.B2, c, optimize=True).reshape(E, -1)


def iproduct_tables(tables, w, dim, phys_weighted):
    """sum over points of tables_d(mode_d, point_d) * w * f for a pre-weighted field."""
    E = phys_weighted.shape[0]
    Q = len(w)
    if dim == 2:
        A0, A1 = tables
        f = phys_weighted.reshape(E, Q, Q) * np.outer(w, w)[None]
        return np.einsum('qj,pi,eji->eqp', A1, A0, f, optimize=True).reshape(E, -1)
    A0, A1, A2 = tables
    ww = w[:, None, None] * w[None, :, None] * w[None, None, :]
    f = phys_weighted.reshape(E, Q, Q, Q) * ww[None]
    return np.einsum('rk,qj,pi,ekji->erqp', A2, A1, A0, f, optimize=True).reshape(E, -1)


def iproduct(basis, dim, jac, phys):
    E = phys.shape[0] if phys.ndim == 2 else phys.size // basis.Q ** dim
    nq = basis.Q ** dim
    phys = phys.reshape(E, nq)
    J = _geo_pts(jac, E, nq)
    return iproduct_tables([basis.B2] * dim, basis.w, dim, J * phys)


def ref_derivs(basis, dim, phys):
    """Derivatives along the reference directions by collocation (PhysDerivTensor*Kernel)."""
    Q = basis.Q
    D2 = basis.D2
    E = phys.size // Q ** dim
    if dim == 2:
        u = phys.reshape(E, Q, Q)
        d0 = np.einsum('ab,ejb->eja', D2, u)
        d1 = np.einsum('ab,ebi->eai', D2, u)
        return [d0.reshape(E, -1), d1.reshape(E, -1)]
    u = phys.reshape(E, Q, Q, Q)
    d0 = np.einsum('ab,ekjb->ekja', D2, u)
    d1 = np.einsum('ab,ekbi->ekai', D2, u)
    d2 = np.einsum('ab,ebji->eaji', D2, u)
    return [d0.reshape(E, -1), d1.reshape(E, -1), d2.reshape(E, -1)]


def physderiv(basis, dim, df, phys):
    """Physical derivatives du/dx_k = sum_j df[k*d+j] du/dxi_j (PhysDerivQuad/HexKernel)."""
    E = phys.size // basis.Q ** dim
    nq = basis.Q ** dim
    d = ref_derivs(basis, dim, phys)
    dfp = _df_pts(df, dim, E, nq)
    return [sum(dfp[k * dim + j] * d[j] for j in range(dim)) for k in range(dim)]


def metric(df, dim, E, nq):
    """Symmetric inverse metric g^{ab} = sum_k df[k*d+a] df[k*d+b] (Helmholtz.h:193-205)."""
    dfp = _df_pts(df, dim, E, nq)
    m = {}
    for a in range(dim):
        for b in range(a, dim):
            m[(a, b)] = sum(dfp[k * dim + a] * dfp[k * dim + b] for k in range(dim))
            m[(b, a)] = m[(a, b)]
    return m


def iproduct_deriv(basis, dim, jac, df, comps):
    """sum_k (d phi / d x_k, comps[k]): IProductWRTDerivBase_IterPerExp
    (Collections/IProductWRTDerivBase.cpp:446-546) forms tmp[j] = sum_k derivFac[j + k d]
    comps[k] (derivFac[j + k d] = df[k*d + j] = d xi_j / d x_k), multiplies by jac and
    takes StdExpansion::IProductWRTDerivBase(j, .), the inner product with the derivative
    table DB in direction j."""
    b = basis
    nq = b.Q ** dim
    E = np.asarray(comps[0]).size // nq
    J = _geo_pts(jac, E, nq)
    dfp = _df_pts(df, dim, E, nq)
    out = 0
    for j in range(dim):
        t = sum(dfp[k * dim + j] * np.asarray(comps[k]).reshape(E, nq) for k in range(dim))
        tables = [b.B2] * dim
        tables[j] = b.DB2
        out = out + iproduct_tables(tables, b.w, dim, J * t)
    return out


def helmholtz(basis, dim, jac, df, lam, coeffs):
    """lambda * M u + L u, composed as HelmholtzQuadImpl / HelmholtzHexImpl."""
    b = basis
    E = coeffs.size // b.n ** dim
    nq = b.Q ** dim
    J = _geo_pts(jac, E, nq)
    bwd = bwdtrans(b, dim, coeffs)
    out = lam * iproduct_tables([b.B2] * dim, b.w, dim, J * bwd)
    d = ref_derivs(b, dim, bwd)
    m = metric(df, dim, E, nq)
    for a in range(dim):
        t = sum(m[(a, c)] * d[c] for c in range(dim))
        tables = [b.B2] * dim
        tables[a] = b.DB2
        out = out + iproduct_tables(tables, b.w, dim, J * t)
    return out


def helmholtz_varcoeff(basis, dim, jac, df, lam, kappa, coeffs):
    """lambda M u + L_kappa u with an isotropic coefficient kappa at quadrature points.

    Restates StdRegions/StdExpansion.cpp:664-717 (LaplacianMatrixOp_MatFree with
    eVarCoeffD00 = eVarCoeffD11 (= D22) = kappa) plus MassMatrixOp (:647-662):
    the Laplacian integrand is kappa * grad(phi) . grad(u).
    """
    b = basis
    E = coeffs.size // b.n ** dim
    nq = b.Q ** dim
    J = _geo_pts(jac, E, nq)
    K = np.asarray(kappa).reshape(E, nq)
    bwd = bwdtrans(b, dim, coeffs)
    out = lam * iproduct_tables([b.B2] * dim, b.w, dim, J * bwd)
    d = ref_derivs(b, dim, bwd)
    m = metric(df, dim, E, nq)
    for a in range(dim):
        t = sum(m[(a, c)] * d[c] for c in range(dim))
        tables = [b.B2] * dim
        tables[a] = b.DB2
        out = out + iproduct_tables(tables, b.w, dim, J * K * t)
    return out


def helmholtz_diag(basis, dim, jac, df, lam):
    """Diagonal of the element Helmholtz matrices, (E, n^d).

    The reference sums the diagonals of dense element matrices
    (MultiRegions/PreconditionerDiagonal.cpp:98-161); the diagonal entry of mode m is
    lambda (phi_m, phi_m)_J + sum_ab (d_a phi_m, g^{ab} d_b phi_m)_J, evaluated here
    by sum factorisation with squared / mixed 1-D tables.
    """
    b = basis
    E = np.asarray(jac).shape[0]
    nq = b.Q ** dim
    J = _geo_pts(jac, E, nq)
    m = metric(df, dim, E, nq)
    BB, DD, BD = b.B2 * b.B2, b.DB2 * b.DB2, b.B2 * b.DB2
    out = lam * iproduct_tables([BB] * dim, b.w, dim, J)
    for a in range(dim):
        for c in range(dim):
            tables = [BB] * dim
            if a == c:
                tables[a] = DD
            else:
                tables[a] = BD
                tables[c] = BD
            out = out + iproduct_tables(tables, b.w, dim, J * m[(a, c)])
    return out



def helmholtz_varcoeff_tensor(basis, dim, jac, df, lam, K, coeffs):
    """lambda M u + sum_{k1,k2} IProductWRTDerivBase(k1, K[k1,k2] du/dx_k2), as
    StdRegions/StdExpansion.cpp:664-717 composes LaplacianMatrixOp_MatFree(k1, k2) with the
    symmetric coefficients eVarCoeffD00, D01, (D02,) D11, (D12, D22) given in K (rows in that
    order, each at the quadrature points)."""
    b = basis
    E = coeffs.size // b.n ** dim
    nq = b.Q ** dim
    J = _geo_pts(jac, E, nq)
    u = bwdtrans(b, dim, coeffs)
    out = lam * iproduct_tables([b.B2] * dim, b.w, dim, J * u)
    d = physderiv(b, dim, df, u)
    Kf = np.asarray(K).reshape(dim * (dim + 1) // 2, E, nq)
    idx, t = {}, 0
    for a in range(dim):
        for c in range(a, dim):
            idx[(a, c)] = idx[(c, a)] = t
            t += 1
    comps = [sum(Kf[idx[(k1, k2)]] * d[k2] for k2 in range(dim)) for k1 in range(dim)]
    return out + iproduct_deriv(b, dim, jac, df, comps)
