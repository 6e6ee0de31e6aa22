"""Geometric factors at quadrature points (oracle restatement).

Follows SpatialDomains/GeomFactors.cpp for coordinate dimension == shape dimension:
  * ComputeDeriv (:168-239): dx_k/dxi_i by collocation differentiation of the
    coordinates held at the quadrature points (map points == target points).
  * ComputeJac (:252-308): g_ij = sum_k dx_k/dxi_i dx_k/dxi_j, J = sqrt(det g).
  * ComputeDerivFactors (:399-475): df[k*d + j] = sum_i dx_k/dxi_i (g^-1)_{ij}
    = dxi_j/dx_k.
and the coalesced layouts of Collections/CoalescedGeomData.cpp:53-313:
``jac[e*nq + q]`` and ``df[dir][e*nq + q]`` for deformed collections.
"""
import numpy as np


def coord_derivs(X, D2, dim):
    """X: (dim, E, Q^dim) coordinates. Returns deriv[i][k] arrays (E, Q^dim)."""
    E = X.shape[1]
    Q = D2.shape[0]
    out = [[None] * dim for _ in range(dim)]
    for k in range(dim):
        if dim == 2:
            x = X[k].reshape(E, Q, Q)  # [e, j, i]
            out[0][k] = np.einsum('ab,ejb->eja', D2, x).reshape(E, -1)
            out[1][k] = np.einsum('ab,ebi->eai', D2, x).reshape(E, -1)
        else:
            x = X[k].reshape(E, Q, Q, Q)  # [e, k, j, i]
            out[0][k] = np.einsum('ab,ekjb->ekja', D2, x).reshape(E, -1)
            out[1][k] = np.einsum('ab,ekbi->ekai', D2, x).reshape(E, -1)
            out[2][k] = np.einsum('ab,ebji->eaji', D2, x).reshape(E, -1)
    return out


def _adjugate(g, dim):
    """Adjugate of the symmetric dim x dim metric (GeomFactors.cpp:718-765, Adjoint)."""
    if dim == 2:
        return [[g[1][1], -g[0][1]], [-g[1][0], g[0][0]]]
    a = [[None] * 3 for _ in range(3)]
    a[0][0] = g[1][1] * g[2][2] - g[1][2] * g[2][1]
    a[0][1] = g[0][2] * g[2][1] - g[0][1] * g[2][2]
    a[0][2] = g[0][1] * g[1][2] - g[0][2] * g[1][1]
    a[1][0] = g[1][2] * g[2][0] - g[1][0] * g[2][2]
    a[1][1] = g[0][0] * g[2][2] - g[0][2] * g[2][0]
    a[1][2] = g[0][2] * g[1][0] - g[0][0] * g[1][2]
    a[2][0] = g[1][0] * g[2][1] - g[1][1] * g[2][0]
    a[2][1] = g[0][1] * g[2][0] - g[0][0] * g[2][1]
    a[2][2] = g[0][0] * g[1][1] - g[0][1] * g[1][0]
    return a


def geom_factors(X, D2, dim):
    """Return (jac (E, nq), df (dim*dim, E*nq)) in the CoalescedGeomData layout."""
    deriv = coord_derivs(X, D2, dim)
    g = [[sum(deriv[i][k] * deriv[j][k] for k in range(dim)) for j in range(dim)]
         for i in range(dim)]
    adj = _adjugate(g, dim)
    det = sum(g[0][i] * adj[i][0] for i in range(dim))
    if np.any(det <= 0.0):
        raise ValueError("non-positive Jacobian (GeomFactors.cpp:610-676 check)")
    ginv = [[adj[i][j] / det for j in range(dim)] for i in range(dim)]
    jac = np.sqrt(det)
    df = np.empty((dim * dim,) + jac.shape)
    for k in range(dim):
        for j in range(dim):
            df[k * dim + j] = sum(deriv[i][k] * ginv[i][j] for i in range(dim))
    E = jac.shape[0]
    return jac, df.reshape(dim * dim, E * jac.shape[1])
