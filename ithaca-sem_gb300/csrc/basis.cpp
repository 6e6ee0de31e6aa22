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
//
// Triangles add direction 1 of the collapsed coordinates:
//   Gauss-Radau-Jacobi points with z_0 = -1, alpha 1, beta 0 (Polylib.cpp:119-144 zwgrjm):
//     interior points the zeros of P_{Q-1}^{(1,1)} (Newton with deflation from
//     Chebyshev-Gauss guesses), weights 2 (1 - z_i) / (Q (Q+1) P_{Q-1}^{(1,0)}(z_i)^2)
//   derivative matrix by the barycentric Lagrange formula (Polylib.cpp:589-626 Dgrjm)
//   ModifiedB modes B1 (n (n+1)/2 of them, q fastest), DB1 = D1 B1 (Basis.cpp:423-507)
// Tetrahedra add direction 2: Gauss-Radau-Jacobi points for the weight (1 - z)^2 and the
// ModifiedC rows phi^c_{pqr} = phi^b_{p+q,r} (Basis.cpp:512-566); pyramids the
// ModifiedPyr_C rows on the same points (Basis.cpp:568-672).
#include "ithaca_internal.h"

#include <algorithm>
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

// Zeros of P_m^{(a,b)}: Newton with deflation from Chebyshev-Gauss guesses.
static void jacobi_zeros(int m, double a, double b, double* x) {
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < m; ++k) {
    double r = -std::cos((2.0 * k + 1.0) * pi / (2.0 * m));
    if (k > 0) r = 0.5 * (r + x[k - 1]);
    for (int it = 0; it < 200; ++it) {
      const double p = jacobi(m, a, b, r);
      const double dp = 0.5 * (m + a + b + 1.0) * jacobi(m - 1, a + 1.0, b + 1.0, r);
      double defl = 0.0;
      for (int j = 0; j < k; ++j) defl += 1.0 / (r - x[j]);
      const double step = p / (dp - p * defl);
      r -= step;
      if (std::fabs(step) < 1e-16) break;
    }
    x[k] = r;
  }
}

// Gauss-Radau-Jacobi points with z_0 = -1 for the weight (1 - z)^alpha: -1 and the zeros
// of P_{Q-1}^{(alpha,1)}; weights 2^alpha (1 - z_i) / (Q (Q + alpha) P_{Q-1}^{(alpha,0)}(z_i)^2).
static void radau_points(int Q, double* z, double* w, double alpha = 1.0) {
  if (Q == 1) { z[0] = 0.0; w[0] = 2.0; return; }
  z[0] = -1.0;
  jacobi_zeros(Q - 1, alpha, 1.0, z + 1);
  for (int i = 0; i < Q; ++i) {
    const double p = jacobi(Q - 1, alpha, 0.0, z[i]);
    w[i] = std::pow(2.0, alpha) * (1.0 - z[i]) / (Q * (Q + alpha) * p * p);
  }
}

// D[k*Q + i] = l_k'(z_i) for any distinct points.
static void lagrange_derivative(int Q, const double* z, double* D) {
  std::vector<double> c(Q, 1.0);
  for (int i = 0; i < Q; ++i)
    for (int j = 0; j < Q; ++j)
      if (j != i) c[i] *= z[i] - z[j];
  for (int i = 0; i < Q; ++i) {
    double diag = 0.0;
    for (int k = 0; k < Q; ++k) {
      if (k == i) continue;
      D[k * Q + i] = c[i] / (c[k] * (z[i] - z[k]));
      diag += 1.0 / (z[i] - z[k]);
    }
    D[i * Q + i] = diag;
  }
}

static void modB_tables(int n, int Q, const double* z, const double* D, double* B, double* DB) {
  int m = 0;
  for (int p = 0; p < n; ++p)
    for (int q = 0; q < n - p; ++q, ++m)
      for (int i = 0; i < Q; ++i) {
        const double lo = 0.5 * (1.0 - z[i]), hi = 0.5 * (1.0 + z[i]);
        double v;
        if (p == 0)
          v = q == 0 ? lo : (q == 1 ? hi : lo * hi * jacobi(q - 2, 1.0, 1.0, z[i]));
        else if (q == 0)
          v = std::pow(lo, p);
        else
          v = std::pow(lo, p) * hi * jacobi(q - 1, 2.0 * p - 1.0, 1.0, z[i]);
        B[m * Q + i] = v;
      }
  for (int mm = 0; mm < m; ++mm)
    for (int i = 0; i < Q; ++i) {
      double s = 0.0;
      for (int k = 0; k < Q; ++k) s += D[k * Q + i] * B[mm * Q + k];
      DB[mm * Q + i] = s;
    }
}

TriBasisTables make_tri_basis(int n) {
  TriBasisTables t;
  t.n = n;
  t.Q0 = n + 1;
  t.Q1 = n;
  t.nc = n * (n + 1) / 2;
  t.a = make_basis(n, n + 1);
  t.z1.resize(t.Q1);
  t.w1.resize(t.Q1);
  t.D1.resize(t.Q1 * t.Q1);
  t.B1.resize((size_t)t.nc * t.Q1);
  t.DB1.resize((size_t)t.nc * t.Q1);
  radau_points(t.Q1, t.z1.data(), t.w1.data());
  lagrange_derivative(t.Q1, t.z1.data(), t.D1.data());
  modB_tables(n, t.Q1, t.z1.data(), t.D1.data(), t.B1.data(), t.DB1.data());
  return t;
}

TetBasisTables make_tet_basis(int n) {
  TetBasisTables t;
  t.n = n;
  t.nc = n * (n + 1) * (n + 2) / 6;
  t.t = make_tri_basis(n);
  const int Q = n, npq = n * (n + 1) / 2;
  t.z2.resize(Q);
  t.w2.resize(Q);
  t.D2.resize(Q * Q);
  radau_points(Q, t.z2.data(), t.w2.data(), 2.0);
  lagrange_derivative(Q, t.z2.data(), t.D2.data());
  // ModifiedC: row (p, q, r) is the ModifiedB row (p + q, r) on the alpha-2 points
  std::vector<double> Bb((size_t)npq * Q), DBb((size_t)npq * Q);
  modB_tables(n, Q, t.z2.data(), t.D2.data(), Bb.data(), DBb.data());
  t.B2.resize((size_t)t.nc * Q);
  t.DB2.resize((size_t)t.nc * Q);
  int m = 0;
  for (int p = 0; p < n; ++p)
    for (int q = 0; q < n - p; ++q)
      for (int r = 0; r < n - p - q; ++r, ++m) {
        int row = r;  // ModifiedB index of (p + q, r)
        for (int pp = 0; pp < p + q; ++pp) row += n - pp;
        for (int k = 0; k < Q; ++k) {
          t.B2[(size_t)m * Q + k] = Bb[(size_t)row * Q + k];
          t.DB2[(size_t)m * Q + k] = DBb[(size_t)row * Q + k];
        }
      }
  return t;
}

PyrBasisTables make_pyr_basis(int n) {
  PyrBasisTables t;
  t.n = n;
  t.nc = n * (n + 1) * (2 * n + 1) / 6;
  t.a = make_basis(n, n + 1);
  const int Q = n, npq = n * (n + 1) / 2;
  t.z2.resize(Q);
  t.w2.resize(Q);
  t.D2.resize(Q * Q);
  radau_points(Q, t.z2.data(), t.w2.data(), 2.0);
  lagrange_derivative(Q, t.z2.data(), t.D2.data());
  std::vector<double> Bb((size_t)npq * Q), DBb((size_t)npq * Q);
  modB_tables(n, Q, t.z2.data(), t.D2.data(), Bb.data(), DBb.data());
  t.B2.resize((size_t)t.nc * Q);
  int m = 0;
  for (int p = 0; p < n; ++p)
    for (int q = 0; q < n; ++q)
      for (int r = 0; r < n - std::max(p, q); ++r, ++m) {
        double* row = &t.B2[(size_t)m * Q];
        if (std::min(p, q) <= 1) {  // the ModifiedB row (max(p, q), r)
          int b = r;
          for (int pp = 0; pp < std::max(p, q); ++pp) b += n - pp;
          for (int k = 0; k < Q; ++k) row[k] = Bb[(size_t)b * Q + k];
        } else {  // ((1-z)/2)^(p+q-2) [(1+z)/2 P_{r-1}^{(2p+2q-3,1)}]
          for (int k = 0; k < Q; ++k) {
            const double z = t.z2[k], lo = 0.5 * (1.0 - z), hi = 0.5 * (1.0 + z);
            row[k] = std::pow(lo, p + q - 2) * (r == 0 ? 1.0 : hi * jacobi(r - 1, 2.0 * p + 2.0 * q - 3.0, 1.0, z));
          }
        }
      }
  t.DB2.resize((size_t)t.nc * Q);
  for (int mm = 0; mm < t.nc; ++mm)
    for (int i = 0; i < Q; ++i) {
      double acc = 0.0;
      for (int k = 0; k < Q; ++k) acc += t.D2[k * Q + i] * t.B2[(size_t)mm * Q + k];
      t.DB2[(size_t)mm * Q + i] = acc;
    }
  return t;
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
