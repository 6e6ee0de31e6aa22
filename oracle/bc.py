"""Boundary-constrained forward transforms (oracle restatement, FP64; test infrastructure).

The reference imposes Dirichlet data through boundary expansions whose coefficients are
boundary-constrained projections of the boundary function:
  segment  StdRegions/StdSegExp.cpp:319-390   vertex modes take the end values, the
           interior modes solve the interior block of the mass matrix against
           IProduct(f) - M (vertex part)
  quad     StdRegions/StdQuadExp.cpp:259-346  the four edges as segments (vertex and edge
           modes), then the interior modes the same way with the 2-D mass matrix
ModifiedA ordering: modes 0, 1 are the vertex modes, 2.. the interior ones; a quad's
coefficient (p, q) is stored at q*n + p and its point (i, j) at j*Q + i.
"""
import numpy as np


def seg_fwd_bnd(basis, f):
    """n coefficients of the boundary-constrained projection of f (Q point values)."""
    B, w, n = basis.B2, basis.w, basis.n
    c = np.zeros(n)
    c[0], c[1] = f[0], f[-1]
    if n > 2:
        M = (B * w) @ B.T
        rhs = B @ (w * f) - M @ c
        c[2:] = np.linalg.solve(M[2:, 2:], rhs[2:])
    return c


def quad_fwd_bnd(basis, f):
    """n*n coefficients (q*n + p) of the boundary-constrained projection of f given at
    the Q*Q points (j*Q + i) of a straight-sided face (constant Jacobian)."""
    n, Q = basis.n, basis.Q
    F = np.asarray(f, dtype=np.float64).reshape(Q, Q)  # F[j, i]
    C = np.zeros((n, n))                               # C[q, p]
    # edges, each projected along increasing coordinate; a reversed traversal (as the
    # reference's edges 2 and 3) re-expresses the same 1-D projection
    C[0, :] = seg_fwd_bnd(basis, F[0, :])    # j = 0:  modes (p, q = 0)
    C[1, :] = seg_fwd_bnd(basis, F[-1, :])   # j = Q-1: modes (p, q = 1)
    C[:, 0] = seg_fwd_bnd(basis, F[:, 0])    # i = 0:  modes (p = 0, q)
    C[:, 1] = seg_fwd_bnd(basis, F[:, -1])   # i = Q-1: modes (p = 1, q)
    if n > 2:
        B, w = basis.B2, basis.w
        M1 = (B * w) @ B.T
        M = np.kron(M1, M1)                            # [(q, p), (q', p')]
        ip = (B @ (F * w[None, :]).T).T                # sum_i B(p, i) w_i F[j, i] -> [j, p]
        ip = B @ (ip * w[:, None])                     # sum_j B(q, j) w_j ...      -> [q, p]
        rhs = ip.reshape(-1) - M @ C.reshape(-1)
        interior = [q * n + p for q in range(2, n) for p in range(2, n)]
        sol = np.linalg.solve(M[np.ix_(interior, interior)], rhs[interior])
        Cf = C.reshape(-1)
        Cf[interior] = sol
        C = Cf.reshape(n, n)
    return C.reshape(-1)
