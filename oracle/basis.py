"""ModifiedA basis tables (oracle restatement of LibUtilities/Foundations/Basis.cpp:392-421).

Storage follows the reference: ``B[p*Q + i]`` is mode p at point z_i (mode-major,
point fastest); ``DB = D @ B`` column-wise, i.e. DB[p*Q+i] = sum_k D(i,k) B[p*Q+k]
(the Dgemm at Basis.cpp:418-420).
  p = 0 : (1 - z)/2
  p = 1 : (1 + z)/2
  p >= 2: (1 - z)/2 (1 + z)/2 P_{p-2}^{(1,1)}(z)
"""
import numpy as np

from . import polylib


class Basis1D:
    """One direction of a tensor-product expansion: n modes on Q GLL points."""

    def __init__(self, n, Q):
        self.n, self.Q = n, Q
        self.z, self.w = polylib.gll(Q)
        self.D = polylib.gll_d(self.z)
        self.D2 = self.D.reshape(Q, Q).T  # D2[i, k] = l_k'(z_i)
        z = self.z
        B = np.zeros((n, Q))
        B[0] = 0.5 * (1.0 - z)
        if n > 1:
            B[1] = 0.5 * (1.0 + z)
        for p in range(2, n):
            B[p] = polylib.jacobi(p - 2, 1.0, 1.0, z) * B[0] * B[1]
        self.B2 = B                       # B2[p, i]
        self.DB2 = (self.D2 @ B.T).T      # DB2[p, i] = sum_k D(i,k) B(p,k)
        self.B = B.reshape(-1).copy()
        self.DB = self.DB2.reshape(-1).copy()
