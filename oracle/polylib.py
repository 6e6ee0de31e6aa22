"""Gauss-Lobatto-Legendre quadrature and Jacobi polynomials (oracle restatement).

Follows the mathematics behind LibUtilities/Polylib/Polylib.cpp:
  * ``jacobi``   -- three-term recurrence of P_n^{(a,b)} (Polylib.cpp:1034-1111, jacobfd).
  * ``gll``      -- GLL zeros z (end points -1, 1 plus the zeros of P_{Q-2}^{(1,1)})
                    and weights w_i = 2 / (Q (Q-1) P_{Q-1}(z_i)^2) (Polylib.cpp:195-228, zwglj).
  * ``gll_d``    -- collocation derivative matrix, returned flattened in the
                    reference's storage order: ``D[k*Q + i] = l_k'(z_i)`` so that
                    du/dz(z_i) = sum_k D[k*Q+i] u_k (Polylib.cpp:690-730, Dglj, then
                    the column-major copy of LibUtilities/Foundations/GaussPoints.cpp:235).
The zeros are found by Newton iteration from Chebyshev-Gauss-Lobatto guesses
(no eigen-solver), which is a different route to the same points.
"""
import numpy as np


def jacobi(n, a, b, z):
    """P_n^{(a,b)}(z) by the standard three-term recurrence (Polylib.cpp:1075-1092)."""
    z = np.asarray(z, dtype=np.float64)
    p0 = np.ones_like(z)
    if n == 0:
        return p0
    p1 = 0.5 * (a - b + (a + b + 2.0) * z)
    for k in range(2, n + 1):
        apb = a + b
        a1 = 2.0 * k * (k + apb) * (2.0 * k + apb - 2.0)
        a2 = (2.0 * k + apb - 1.0) * (a * a - b * b)
        a3 = (2.0 * k + apb - 2.0) * (2.0 * k + apb - 1.0) * (2.0 * k + apb)
        a4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * (2.0 * k + apb)
        p0, p1 = p1, ((a2 / a1 + a3 / a1 * z) * p1 - a4 / a1 * p0)
    return p1


def _legendre_and_deriv(N, z):
    """Legendre P_N and P_N' (Bonnet recurrence), for the Newton iteration."""
    p_prev = np.ones_like(z)
    if N == 0:
        return p_prev, np.zeros_like(z)
    p = z.copy()
    for k in range(2, N + 1):
        p_prev, p = p, ((2 * k - 1) * z * p - (k - 1) * p_prev) / k
    dp = N * (z * p - p_prev) / (z * z - 1.0)
    return p, dp


def gll(Q):
    """GLL points and weights on [-1, 1] (zwglj with alpha = beta = 0)."""
    if Q == 1:
        return np.zeros(1), np.full(1, 2.0)
    if Q == 2:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    N = Q - 1
    z = -np.cos(np.pi * np.arange(Q) / N)
    # Newton on q(z) = (1 - z^2) P_N'(z), whose zeros are exactly the GLL points.
    zi = z[1:-1].copy()
    for _ in range(100):
        p, dp = _legendre_and_deriv(N, zi)
        # (1-z^2) P_N'' = 2 z P_N' - N(N+1) P_N  =>  q' = -N(N+1) P_N
        q = (1.0 - zi * zi) * dp
        dq = -N * (N + 1) * p
        step = q / dq
        zi -= step
        if np.max(np.abs(step)) < 1e-16:
            break
    z[1:-1] = zi
    z[0], z[-1] = -1.0, 1.0
    pN = jacobi(N, 0.0, 0.0, z)
    w = 2.0 / (N * (N + 1) * pN * pN)
    return z, w


def gll_d(z):
    """Flattened collocation derivative matrix, D[k*Q + i] = l_k'(z_i)."""
    Q = len(z)
    D2 = np.zeros((Q, Q))  # D2[i, k] = l_k'(z_i)
    if Q <= 1:
        return D2.reshape(-1)
    N = Q - 1
    pN = jacobi(N, 0.0, 0.0, z)
    for i in range(Q):
        for k in range(Q):
            if i != k:
                D2[i, k] = pN[i] / (pN[k] * (z[i] - z[k]))
    D2[0, 0] = -N * (N + 1) / 4.0
    D2[N, N] = N * (N + 1) / 4.0
    # column-major flattening: element (i, k) stored at k*Q + i
    return D2.T.reshape(-1).copy()
