// Host construction of the 1-D tables of the ModifiedA / Gauss-Lobatto-Legendre basis.
//
// Same quantities as the reference (written from the mathematics, not translated):
//   GLL points z and weights w   -- LibUtilities/Polylib/Polylib.cpp:195-228 (zwglj)
//   derivative matrix D          -- Polylib.cpp:690-730 (Dglj), stored as the reference's
//                                   column-major NekMatrix (GaussPoints.cpp:235):
//                                   D[k*Q + i] = l_k'(z_i)
//   ModifiedA modes B, DB = D B  -- LibUtilities/Foundations/Basis.cpp:392-421
// Points: Newton iteration on (1 - z^2) P'_{Q-1}(z) from Chebyshev-Gauss-Lobatto
// guesses; weights 2 / (Q (Q-1) P_{Q-1}(z)^2); D by the Lagrange-derivative formula.
#include "ithaca_internal.h"

#include <cmath>

namespace ithaca {

// Jacobi polynomial P_m^{(a,b)}(x) by the three-term recurrence.
double jacobi(int m, double a, double b, double x) {
  if (m == 0) return 1.0;
  double p0 = 1.0, p1 = 0.5 * (a - b + (a + b + 2.0) * x);
  for (int k = 2; k <= m; ++k) {
    const double apb = a + b;
    const double a1 = 2.0 * k * (k + apb) * (2.0 * k + apb - 2.0);
    const double a2 = (2.0 * k + apb - 1.0) * (a * a - b * b);
    const double a3 = (2.0 * k + apb - 2.0) * (2.0 * k + apb - 1.0) * (2.0 * k + apb);
    const double a4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * (2.0 * k + apb);
    const double p2 = ((a2 / a1 + a3 / a1 * x) * p1 - a4 / a1 * p0);
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

static void legendre_pd(int N, double x, double* p, double* dp) {
  double pm = 1.0, pc = x;
  if (N == 0) { *p = 1.0; *dp = 0.0; return; }
  for (int k = 2; k <= N; ++k) {
    double pn = ((2 * k - 1) * x * pc - (k - 1) * pm) / k;
    pm = pc;
    pc = pn;
  }
  *p = pc;
  *dp = N * (x * pc - pm) / (x * x - 1.0);
}

void gll_points(int Q, double* z, double* w) {
  if (Q == 1) { z[0] = 0.0; w[0] = 2.0; return; }
  const int N = Q - 1;
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < Q; ++i) z[i] = -std::cos(pi * i / N);
  for (int i = 1; i < N; ++i) {
    double x = z[i];
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre_pd(N, x, &p, &dp);
      const double q = (1.0 - x * x) * dp;
      const double dq = -N * (N + 1.0) * p;
      const double step = q / dq;
      x -= step;
      if (std::fabs(step) < 1e-16) break;
    }
    z[i] = x;
  }
  z[0] = -1.0;
  z[N] = 1.0;
  for (int i = 0; i < Q; ++i) {
    const double pN = jacobi(N, 0.0, 0.0, z[i]);
    w[i] = 2.0 / (N * (N + 1.0) * pN * pN);
  }
}

void gll_derivative(int Q, const double* z, double* D) {
  const int N = Q - 1;
  for (int i = 0; i < Q; ++i)
    for (int k = 0; k < Q; ++k) {
      double v = 0.0;
      if (i != k) {
        v = jacobi(N, 0, 0, z[i]) / (jacobi(N, 0, 0, z[k]) * (z[i] - z[k]));
      } else if (i == 0 && Q > 1) {
        v = -N * (N + 1.0) / 4.0;
      } else if (i == N && Q > 1) {
        v = N * (N + 1.0) / 4.0;
      }
      D[k * Q + i] = v;
    }
}

void modA_tables(int n, int Q, const double* z, const double* D, double* B, double* DB) {
  for (int i = 0; i < Q; ++i) {
    B[i] = 0.5 * (1.0 - z[i]);
    if (n > 1) B[Q + i] = 0.5 * (1.0 + z[i]);
  }
  for (int p = 2; p < n; ++p)
    for (int i = 0; i < Q; ++i) B[p * Q + i] = jacobi(p - 2, 1.0, 1.0, z[i]) * B[i] * B[Q + i];
  for (int p = 0; p < n; ++p)
    for (int i = 0; i < Q; ++i) {
      double s = 0.0;
      for (int k = 0; k < Q; ++k) s += D[k * Q + i] * B[p * Q + k];
      DB[p * Q + i] = s;
    }
}

BasisTables make_basis(int n, int Q) {
  BasisTables t;
  t.n = n;
  t.Q = Q;
  t.z.resize(Q);
  t.w.resize(Q);
  t.D.resize(Q * Q);
  t.B.resize(n * Q);
  t.DB.resize(n * Q);
  gll_points(Q, t.z.data(), t.w.data());
  gll_derivative(Q, t.z.data(), t.D.data());
  modA_tables(n, Q, t.z.data(), t.D.data(), t.B.data(), t.DB.data());
  return t;
}

}  // namespace ithaca
