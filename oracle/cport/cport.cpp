// Compiled CPU port of the reference Helmholtz + CG path (TEST INFRASTRUCTURE / CPU BASELINE).
//
// A C++ restatement, in this project's own code, of the arithmetic of
//   MatrixFreeOps/Helmholtz.h:137-275 (HelmholtzQuadImpl) and :763-993 (HelmholtzHexImpl),
//   built from the sum-factorisation kernels of MatrixFreeOps/BwdTransKernels.hpp:35-76,302-372,
//   IProductKernels.hpp:76-133,236-314 and PhysDerivKernels.hpp:39-151,219-374;
//   AssemblyMapCG::GlobalToLocal / Assemble (MultiRegions/AssemblyMap/AssemblyMapCG.cpp:2853-2910);
//   NekLinSysIterCG::DoConjugateGradient (LibUtilities/LinearAlgebra/NekLinSysIterCG.cpp:104-263).
// It keeps the reference's operation count (separate BwdTrans, mass IProduct, collocation
// derivatives, metric, and d derivative IProducts with DB) and runs one std::thread per
// core over contiguous element / dof ranges, standing in for the reference's MPI ranks.
// It exists because the reference tree is not available where the CPU baseline is timed;
// where it is, oracle/_ref (the reference kernels compiled in place) pins this port.
// Triangles: cport_tri_helmholtz restates HelmholtzTriImpl (MatrixFreeOps/Helmholtz.h:
// 505-635) on tables passed in by the caller (the oracle's TriBasis).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ---- tables: ModifiedA on GLL, same storage as the reference (B[p*Q+i], D[k*Q+i]) ----
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

struct Tab {
  int n, Q;
  std::vector<double> z, w, D, B, DB;
  Tab(int n_, int Q_) : n(n_), Q(Q_), z(Q_), w(Q_), D(Q_ * Q_), B(n_ * Q_), DB(n_ * Q_) {
    const int N = Q - 1;
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < Q; ++i) z[i] = -std::cos(pi * i / N);
    for (int i = 1; i < N; ++i) {
      double x = z[i];
      for (int it = 0; it < 100; ++it) {
        double pm = 1.0, pc = x;
        for (int k = 2; k <= N; ++k) {
          double pn = ((2 * k - 1) * x * pc - (k - 1) * pm) / k;
          pm = pc;
          pc = pn;
        }
        const double dp = N * (x * pc - pm) / (x * x - 1.0);
        const double step = (1.0 - x * x) * dp / (-N * (N + 1.0) * pc);
        x -= step;
        if (std::fabs(step) < 1e-16) break;
      }
      z[i] = x;
    }
    z[0] = -1.0;
    z[N] = 1.0;
    for (int i = 0; i < Q; ++i) {
      const double pN = jacobi(N, 0, 0, z[i]);
      w[i] = 2.0 / (N * (N + 1.0) * pN * pN);
    }
    for (int i = 0; i < Q; ++i)
      for (int k = 0; k < Q; ++k) {
        double v = 0;
        if (i != k) v = jacobi(N, 0, 0, z[i]) / (jacobi(N, 0, 0, z[k]) * (z[i] - z[k]));
        else if (i == 0) v = -N * (N + 1.0) / 4.0;
        else if (i == N) v = N * (N + 1.0) / 4.0;
        D[k * Q + i] = v;
      }
    for (int i = 0; i < Q; ++i) {
      B[i] = 0.5 * (1 - z[i]);
      B[Q + i] = 0.5 * (1 + z[i]);
    }
    for (int p = 2; p < n; ++p)
      for (int i = 0; i < Q; ++i) B[p * Q + i] = jacobi(p - 2, 1, 1, z[i]) * B[i] * B[Q + i];
    for (int p = 0; p < n; ++p)
      for (int i = 0; i < Q; ++i) {
        double s = 0;
        for (int k = 0; k < Q; ++k) s += D[k * Q + i] * B[p * Q + k];
        DB[p * Q + i] = s;
      }
  }
};

// ---- quad element operator, reference composition ----
template <int N, int Q>
struct QuadOp {
  // u[j*Q+i] = sum_q B1[q,j] sum_p B0[p,i] c[q*N+p]
  static void bwd(const double* B, const double* c, double* u) {
    double t[Q * N];
    for (int i = 0; i < Q; ++i)
      for (int q = 0; q < N; ++q) {
        double s = 0;
        for (int p = 0; p < N; ++p) s += c[q * N + p] * B[p * Q + i];
        t[i * N + q] = s;
      }
    for (int j = 0; j < Q; ++j)
      for (int i = 0; i < Q; ++i) {
        double s = 0;
        for (int q = 0; q < N; ++q) s += t[i * N + q] * B[q * Q + j];
        u[j * Q + i] = s;
      }
  }
  // out[q*N+p] (=|+=) scale * sum_j A1[q,j] w_j sum_i A0[p,i] w_i J u
  static void ipr(const double* A0, const double* A1, const double* w, const double* jac, bool def,
                  const double* u, double* out, double scale, bool append) {
    double sj[Q];
    for (int p = 0; p < N; ++p) {
      for (int j = 0; j < Q; ++j) {
        double s = 0;
        for (int i = 0; i < Q; ++i) s += u[j * Q + i] * A0[p * Q + i] * (def ? jac[j * Q + i] : jac[0]) * w[i];
        sj[j] = s;
      }
      for (int q = 0; q < N; ++q) {
        double s = 0;
        for (int j = 0; j < Q; ++j) s += sj[j] * A1[q * Q + j] * w[j];
        out[q * N + p] = append ? out[q * N + p] + scale * s : scale * s;
      }
    }
  }
  // single operators of one element (BwdTrans, IProductWRTBase, PhysDeriv)
  static void bwd_e(const Tab& t, const double* c, double* u) { bwd(t.B.data(), c, u); }
  static void ipr_e(const Tab& t, const double* jac, bool def, const double* u, double* out) {
    ipr(t.B.data(), t.B.data(), t.w.data(), jac, def, u, out, 1.0, false);
  }
  // du/dx_k = sum_j df[k*2+j] du/dxi_j (collocation derivatives, PhysDerivQuadKernel)
  static void deriv_e(const Tab& t, const double* df, bool def, const double* u, double* const* d) {
    const double* D = t.D.data();
    for (int j = 0; j < Q; ++j)
      for (int i = 0; i < Q; ++i) {
        double a = 0, b = 0;
        for (int k = 0; k < Q; ++k) {
          a += D[k * Q + i] * u[j * Q + k];
          b += u[k * Q + i] * D[k * Q + j];
        }
        const int c = j * Q + i;
        const double* f = def ? df + 4 * c : df;
        d[0][c] = f[0] * a + f[1] * b;
        d[1][c] = f[2] * a + f[3] * b;
      }
  }
  static void apply(const Tab& t, const double* jac, const double* df, bool def, double lam, const double* in,
                    double* out) {
    constexpr int nq = Q * Q;
    double u[nq], d0[nq], d1[nq];
    bwd(t.B.data(), in, u);
    ipr(t.B.data(), t.B.data(), t.w.data(), jac, def, u, out, lam, false);
    const double* D = t.D.data();
    for (int j = 0; j < Q; ++j)
      for (int i = 0; i < Q; ++i) {
        double a = 0, b = 0;
        for (int k = 0; k < Q; ++k) {
          a += D[k * Q + i] * u[j * Q + k];
          b += u[k * Q + i] * D[k * Q + j];
        }
        d0[j * Q + i] = a;
        d1[j * Q + i] = b;
      }
    for (int c = 0; c < nq; ++c) {
      const double* f = def ? df + 4 * c : df;
      const double m00 = f[0] * f[0] + f[2] * f[2], m01 = f[0] * f[1] + f[2] * f[3], m11 = f[1] * f[1] + f[3] * f[3];
      const double a = d0[c], b = d1[c];
      u[c] = m00 * a + m01 * b;
      d0[c] = m01 * a + m11 * b;
    }
    ipr(t.DB.data(), t.B.data(), t.w.data(), jac, def, u, out, 1.0, true);
    ipr(t.B.data(), t.DB.data(), t.w.data(), jac, def, d0, out, 1.0, true);
  }
};

// ---- hex element operator, reference composition ----
template <int N, int Q>
struct HexOp {
  static void bwd(const double* B, const double* c, double* u) {
    double s1[Q * N * N], s2[Q * Q * N];
    for (int i = 0; i < Q; ++i)
      for (int r = 0; r < N; ++r)
        for (int q = 0; q < N; ++q) {
          double s = 0;
          for (int p = 0; p < N; ++p) s += c[(r * N + q) * N + p] * B[p * Q + i];
          s1[(i * N + r) * N + q] = s;
        }
    for (int j = 0; j < Q; ++j)
      for (int i = 0; i < Q; ++i)
        for (int r = 0; r < N; ++r) {
          double s = 0;
          for (int q = 0; q < N; ++q) s += s1[(i * N + r) * N + q] * B[q * Q + j];
          s2[(j * Q + i) * N + r] = s;
        }
    for (int k = 0; k < Q; ++k)
      for (int j = 0; j < Q; ++j)
        for (int i = 0; i < Q; ++i) {
          double s = 0;
          for (int r = 0; r < N; ++r) s += s2[(j * Q + i) * N + r] * B[r * Q + k];
          u[(k * Q + j) * Q + i] = s;
        }
  }
  static void ipr(const double* A0, const double* A1, const double* A2, const double* w, const double* jac, bool def,
                  const double* u, double* out, double scale, bool append) {
    double skj[Q * Q], sk[Q];
    for (int p = 0; p < N; ++p) {
      for (int k = 0; k < Q; ++k)
        for (int j = 0; j < Q; ++j) {
          double s = 0;
          for (int i = 0; i < Q; ++i) {
            const int c = (k * Q + j) * Q + i;
            s += u[c] * A0[p * Q + i] * (def ? jac[c] : jac[0]) * w[i];
          }
          skj[k * Q + j] = s;
        }
      for (int q = 0; q < N; ++q) {
        for (int k = 0; k < Q; ++k) {
          double s = 0;
          for (int j = 0; j < Q; ++j) s += skj[k * Q + j] * A1[q * Q + j] * w[j];
          sk[k] = s;
        }
        for (int r = 0; r < N; ++r) {
          double s = 0;
          for (int k = 0; k < Q; ++k) s += sk[k] * A2[r * Q + k] * w[k];
          const int o = (r * N + q) * N + p;
          out[o] = append ? out[o] + scale * s : scale * s;
        }
      }
    }
  }
  static void bwd_e(const Tab& t, const double* c, double* u) { bwd(t.B.data(), c, u); }
  static void ipr_e(const Tab& t, const double* jac, bool def, const double* u, double* out) {
    ipr(t.B.data(), t.B.data(), t.B.data(), t.w.data(), jac, def, u, out, 1.0, false);
  }
  // du/dx_k = sum_j df[k*3+j] du/dxi_j (collocation derivatives, PhysDerivHexKernel)
  static void deriv_e(const Tab& t, const double* df, bool def, const double* u, double* const* d) {
    const double* D = t.D.data();
    for (int k = 0; k < Q; ++k)
      for (int j = 0; j < Q; ++j)
        for (int i = 0; i < Q; ++i) {
          double a = 0, b = 0, c = 0;
          for (int m = 0; m < Q; ++m) {
            a += D[m * Q + i] * u[(k * Q + j) * Q + m];
            b += u[(k * Q + m) * Q + i] * D[m * Q + j];
            c += u[(m * Q + j) * Q + i] * D[m * Q + k];
          }
          const int o = (k * Q + j) * Q + i;
          const double* f = def ? df + 9 * o : df;
          d[0][o] = f[0] * a + f[1] * b + f[2] * c;
          d[1][o] = f[3] * a + f[4] * b + f[5] * c;
          d[2][o] = f[6] * a + f[7] * b + f[8] * c;
        }
  }
  static void apply(const Tab& t, const double* jac, const double* df, bool def, double lam, const double* in,
                    double* out) {
    constexpr int nq = Q * Q * Q;
    static thread_local std::vector<double> buf(4 * nq);
    if ((int)buf.size() < 4 * nq) buf.resize(4 * nq);
    double *u = buf.data(), *d0 = u + nq, *d1 = d0 + nq, *d2 = d1 + nq;
    const double *B = t.B.data(), *DB = t.DB.data(), *D = t.D.data(), *w = t.w.data();
    bwd(B, in, u);
    ipr(B, B, B, w, jac, def, u, out, lam, false);
    for (int k = 0; k < Q; ++k)
      for (int j = 0; j < Q; ++j)
        for (int i = 0; i < Q; ++i) {
          double a = 0, b = 0, c = 0;
          for (int m = 0; m < Q; ++m) {
            a += D[m * Q + i] * u[(k * Q + j) * Q + m];
            b += u[(k * Q + m) * Q + i] * D[m * Q + j];
            c += u[(m * Q + j) * Q + i] * D[m * Q + k];
          }
          const int o = (k * Q + j) * Q + i;
          d0[o] = a;
          d1[o] = b;
          d2[o] = c;
        }
    for (int c = 0; c < nq; ++c) {
      const double* f = def ? df + 9 * c : df;
      const double m00 = f[0] * f[0] + f[3] * f[3] + f[6] * f[6];
      const double m01 = f[0] * f[1] + f[3] * f[4] + f[6] * f[7];
      const double m02 = f[0] * f[2] + f[3] * f[5] + f[6] * f[8];
      const double m11 = f[1] * f[1] + f[4] * f[4] + f[7] * f[7];
      const double m12 = f[1] * f[2] + f[4] * f[5] + f[7] * f[8];
      const double m22 = f[2] * f[2] + f[5] * f[5] + f[8] * f[8];
      const double a = d0[c], b = d1[c], cc = d2[c];
      d0[c] = m00 * a + m01 * b + m02 * cc;
      d1[c] = m01 * a + m11 * b + m12 * cc;
      d2[c] = m02 * a + m12 * b + m22 * cc;
    }
    ipr(DB, B, B, w, jac, def, d0, out, 1.0, true);
    ipr(B, DB, B, w, jac, def, d1, out, 1.0, true);
    ipr(B, B, DB, w, jac, def, d2, out, 1.0, true);
  }
};

using ApplyFn = void (*)(const Tab&, const double*, const double*, bool, double, const double*, double*);
using BwdFn = void (*)(const Tab&, const double*, double*);
using IprFn = void (*)(const Tab&, const double*, bool, const double*, double*);
using DerivFn = void (*)(const Tab&, const double*, bool, const double*, double* const*);
struct ElemFns {
  BwdFn bwd;
  IprFn ipr;
  DerivFn deriv;
};

ElemFns pick_elem(int dim, int n, int Q) {
#define P(NN, QQ)                                                                           \
  if (n == NN && Q == QQ)                                                                   \
    return dim == 2 ? ElemFns{&QuadOp<NN, QQ>::bwd_e, &QuadOp<NN, QQ>::ipr_e, &QuadOp<NN, QQ>::deriv_e} \
                    : ElemFns{&HexOp<NN, QQ>::bwd_e, &HexOp<NN, QQ>::ipr_e, &HexOp<NN, QQ>::deriv_e};
  P(2, 3) P(3, 4) P(4, 5) P(5, 6) P(6, 7) P(7, 8) P(8, 9) P(9, 10) P(10, 11)
#undef P
  return ElemFns{nullptr, nullptr, nullptr};
}

ApplyFn pick(int dim, int n, int Q) {
#define P(NN, QQ) \
  if (n == NN && Q == QQ) return dim == 2 ? &QuadOp<NN, QQ>::apply : &HexOp<NN, QQ>::apply;
  P(2, 3) P(3, 4) P(4, 5) P(5, 6) P(6, 7) P(7, 8) P(8, 9) P(9, 10) P(10, 11)
#undef P
  return nullptr;
}

template <class F>
void parallel(long long n, int nth, F f) {
  nth = std::max(1, (int)std::min<long long>(nth, n));
  if (nth == 1) {
    f(0, n, 0);
    return;
  }
  std::vector<std::thread> th;
  const long long chunk = (n + nth - 1) / nth;
  for (int t = 0; t < nth; ++t) {
    const long long a = t * chunk, b = std::min(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([=] { f(a, b, t); });
  }
  for (auto& x : th) x.join();
}

// Per-element geometry in the reference's interleave-free layout: jac[e*nq+q] / df[(e*nq+q)*d*d + dir].
struct Geo {
  std::vector<double> jac, df;
};

Geo regroup(int dim, int nq, int E, bool def, const double* jac, const double* df) {
  const int ndf = dim * dim, npt = def ? nq : 1;
  Geo g;
  g.jac.assign(jac, jac + (size_t)E * npt);
  g.df.resize((size_t)E * npt * ndf);
  for (int e = 0; e < E; ++e)
    for (int q = 0; q < npt; ++q)
      for (int d = 0; d < ndf; ++d) g.df[((size_t)e * npt + q) * ndf + d] = df[(size_t)d * E * npt + (size_t)e * npt + q];
  return g;
}


// ---- triangles: HelmholtzTriImpl (MatrixFreeOps/Helmholtz.h:505-635) with CORRECT ----
// Tables (caller's, reference storage): B0/DB0 [p*Q0+i], D0 [k*Q0+i], w0, z0; B1/DB1
// [m*Q1+j] (m(p,q), q fastest), D1 [l*Q1+j], w1 (as GetW(), the factor 1/2 applied here), z1.
struct TriTab {
  int n, Q0, Q1, nc;
  const double *B0, *DB0, *D0, *w0, *z0, *B1, *DB1, *D1, *w1, *z1;
};

// IProductTriKernel: out[m] (+)= sum_j A1[m][j] w1[j] sum_i A0[p][i] w0[i] J f[j][i], CORRECT term to m = 1.
static void tri_ipr(const TriTab& t, const double* A0, const double* A1, const double* f, const double* J,
                    bool def, double scale, bool append, double* out, double* wsp) {
  const int n = t.n, Q0 = t.Q0, Q1 = t.Q1;
  for (int m = 0, p = 0; p < n; ++p) {
    for (int j = 0; j < Q1; ++j) {
      double s = 0;
      for (int i = 0; i < Q0; ++i) s += f[j * Q0 + i] * A0[p * Q0 + i] * (def ? J[j * Q0 + i] : J[0]) * t.w0[i];
      wsp[j] = s;
    }
    for (int q = 0; q < n - p; ++q, ++m) {
      double s = 0;
      for (int j = 0; j < Q1; ++j) s += wsp[j] * A1[m * Q1 + j] * 0.5 * t.w1[j];
      out[m] = append ? out[m] + scale * s : scale * s;
    }
  }
  double c = 0;
  for (int j = 0; j < Q1; ++j)
    for (int i = 0; i < Q0; ++i)
      c += f[j * Q0 + i] * 0.5 * t.w1[j] * A1[Q1 + j] * t.w0[i] * (def ? J[j * Q0 + i] : J[0]) * A0[Q0 + i];
  out[1] += scale * c;
}

static void tri_helm_elem(const TriTab& t, const double* J, const double* df, bool def, double lambda,
                          const double* in, double* out, std::vector<double>& ws) {
  const int n = t.n, Q0 = t.Q0, Q1 = t.Q1, nq = Q0 * Q1;
  double* u = ws.data();
  double* d0 = u + nq;
  double* d1 = d0 + nq;
  double* ps = d1 + nq;  // n * Q1, also IProduct scratch
  // BwdTransTriKernel
  for (int j = 0; j < Q1; ++j) {
    for (int p = 0, m = 0; p < n; ++p) {
      double s = 0;
      for (int q = 0; q < n - p; ++q, ++m) s += t.B1[m * Q1 + j] * in[m];
      ps[p] = s;
    }
    for (int i = 0; i < Q0; ++i) {
      double s = 0;
      for (int p = 0; p < n; ++p) s += ps[p] * t.B0[p * Q0 + i];
      s += in[1] * t.B0[Q0 + i] * t.B1[Q1 + j];
      u[j * Q0 + i] = s;
    }
  }
  tri_ipr(t, t.B0, t.B1, u, J, def, lambda, false, out, ps);
  // PhysDerivTensor2DKernel + the collapsed metric
  for (int j = 0; j < Q1; ++j)
    for (int i = 0; i < Q0; ++i) {
      double a = 0, b = 0;
      for (int k = 0; k < Q0; ++k) a += t.D0[k * Q0 + i] * u[j * Q0 + k];
      for (int k = 0; k < Q1; ++k) b += t.D1[k * Q1 + j] * u[k * Q0 + i];
      d0[j * Q0 + i] = a;
      d1[j * Q0 + i] = b;
    }
  for (int j = 0, c = 0; j < Q1; ++j) {
    const double h1 = 2.0 / (1.0 - t.z1[j]);
    for (int i = 0; i < Q0; ++i, ++c) {
      const double* f = def ? df + (size_t)c * 4 : df;
      const double h0 = 0.5 * (1.0 + t.z0[i]);
      const double a = h1 * (f[0] + h0 * f[1]), b = h1 * (f[2] + h0 * f[3]);
      const double m00 = a * a + b * b, m01 = a * f[1] + b * f[3], m11 = f[1] * f[1] + f[3] * f[3];
      const double x = d0[c], y = d1[c];
      u[c] = m00 * x + m01 * y;
      d0[c] = m01 * x + m11 * y;
    }
  }
  tri_ipr(t, t.DB0, t.B1, u, J, def, 1.0, true, out, ps);
  tri_ipr(t, t.B0, t.DB1, d0, J, def, 1.0, true, out, ps);
}
}  // namespace

extern "C" {

// Triangle Helmholtz apply (E elements, n modes, Q0 = n + 1, Q1 = n); geometry in the
// reference layouts jac[e*nq + q] / df[dir][e*nq + q] (deformed) or per element.
int cport_tri_helmholtz(int n, int E, const double* B0, const double* DB0, const double* D0, const double* w0,
                        const double* z0, const double* B1, const double* DB1, const double* D1, const double* w1,
                        const double* z1, const double* jac, const double* df, int deformed, double lambda,
                        const double* in, double* out, int nthreads) {
  if (n < 2) return 1;
  TriTab t{n, n + 1, n, n * (n + 1) / 2, B0, DB0, D0, w0, z0, B1, DB1, D1, w1, z1};
  const int nq = t.Q0 * t.Q1, npt = deformed ? nq : 1;
  Geo g = regroup(2, nq, E, deformed != 0, jac, df);
  parallel(E, nthreads, [&](long long a, long long b, int) {
    std::vector<double> ws(3 * nq + n * t.Q1 + t.Q1);
    for (long long e = a; e < b; ++e)
      tri_helm_elem(t, &g.jac[e * npt], &g.df[e * npt * 4], deformed != 0, lambda, in + e * t.nc, out + e * t.nc,
                    ws);
  });
  return 0;
}

int cport_helmholtz(int dim, int n, int Q, int E, const double* jac, const double* df, int deformed, double lambda,
                    const double* in, double* out, int nthreads) {
  ApplyFn f = pick(dim, n, Q);
  if (!f) return 1;
  Tab t(n, Q);
  const int nm = dim == 2 ? n * n : n * n * n, nq = dim == 2 ? Q * Q : Q * Q * Q, npt = deformed ? nq : 1;
  Geo g = regroup(dim, nq, E, deformed != 0, jac, df);
  parallel(E, nthreads, [&](long long a, long long b, int) {
    for (long long e = a; e < b; ++e)
      f(t, &g.jac[e * npt], &g.df[e * npt * dim * dim], deformed != 0, lambda, in + e * nm, out + e * nm);
  });
  return 0;
}

// BwdTrans: coefficients (E n^d) -> physical values (E Q^d).
int cport_bwdtrans(int dim, int n, int Q, int E, const double* in, double* out, int nthreads) {
  ElemFns f = pick_elem(dim, n, Q);
  if (!f.bwd) return 1;
  Tab t(n, Q);
  const int nm = dim == 2 ? n * n : n * n * n, nq = dim == 2 ? Q * Q : Q * Q * Q;
  parallel(E, nthreads, [&](long long a, long long b, int) {
    for (long long e = a; e < b; ++e) f.bwd(t, in + e * nm, out + e * nq);
  });
  return 0;
}

// IProductWRTBase: physical values -> coefficients, weighted by J w.
int cport_iproduct(int dim, int n, int Q, int E, const double* jac, int deformed, const double* in, double* out,
                   int nthreads) {
  ElemFns f = pick_elem(dim, n, Q);
  if (!f.ipr) return 1;
  Tab t(n, Q);
  const int nm = dim == 2 ? n * n : n * n * n, nq = dim == 2 ? Q * Q : Q * Q * Q, npt = deformed ? nq : 1;
  parallel(E, nthreads, [&](long long a, long long b, int) {
    for (long long e = a; e < b; ++e) f.ipr(t, jac + e * npt, deformed != 0, in + e * nq, out + e * nm);
  });
  return 0;
}

// PhysDeriv: physical values -> d arrays of physical derivatives (d2 unused in 2-D).
int cport_physderiv(int dim, int n, int Q, int E, const double* df, int deformed, const double* in, double* d0,
                    double* d1, double* d2, int nthreads) {
  ElemFns f = pick_elem(dim, n, Q);
  if (!f.deriv) return 1;
  Tab t(n, Q);
  const int nq = dim == 2 ? Q * Q : Q * Q * Q, npt = deformed ? nq : 1;
  Geo g = regroup(dim, nq, E, deformed != 0, df, df);  // jac unused: df regrouped per point
  const int ndf = dim * dim;
  parallel(E, nthreads, [&](long long a, long long b, int) {
    for (long long e = a; e < b; ++e) {
      double* d[3] = {d0 + e * nq, d1 + e * nq, dim == 3 ? d2 + e * nq : nullptr};
      f.deriv(t, &g.df[e * npt * ndf], deformed != 0, in + e * nq, d);
    }
  });
  return 0;
}

// Reference CG recurrence with Jacobi preconditioning around the element operator;
// returns iterations (>= 0), -1 past max_iter, -2 on a bad (n, Q).
int cport_cg_solve(int dim, int n, int Q, int E, const double* jac, const double* df, int deformed, double lambda,
                   const int* l2g, const double* sign, int nglobal, int ndir, const double* dinv, const double* rhs,
                   double* x, double tol, int max_iter, int nthreads, double* final_eps) {
  ApplyFn f = pick(dim, n, Q);
  if (!f) return -2;
  Tab t(n, Q);
  const int nm = dim == 2 ? n * n : n * n * n, nq = dim == 2 ? Q * Q : Q * Q * Q, npt = deformed ? nq : 1;
  Geo g = regroup(dim, nq, E, deformed != 0, jac, df);
  const long long nloc = (long long)E * nm;
  const int nnd = nglobal - ndir;
  // CSR of the assembly (owner computes; threads own global-dof ranges)
  std::vector<int> rowptr(nglobal + 1, 0), col(nloc);
  for (long long l = 0; l < nloc; ++l) rowptr[l2g[l] + 1]++;
  for (int i = 0; i < nglobal; ++i) rowptr[i + 1] += rowptr[i];
  {
    std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
    for (long long l = 0; l < nloc; ++l) col[fill[l2g[l]]++] = (int)l;
  }
  std::vector<double> wA(nglobal, 0.0), sA(nglobal, 0.0), p(nnd, 0.0), r(nnd), q(nnd, 0.0), li(nloc), lo(nloc);
  std::vector<double> part(3 * std::max(1, nthreads));
  auto apply = [&](const std::vector<double>& gin, std::vector<double>& gout) {
    parallel(E, nthreads, [&](long long a, long long b, int) {
      for (long long e = a; e < b; ++e) {
        for (int m = 0; m < nm; ++m) {
          const long long l = e * nm + m;
          li[l] = sign[l] * gin[l2g[l]];
        }
        f(t, &g.jac[e * npt], &g.df[e * npt * dim * dim], deformed != 0, lambda, &li[e * nm], &lo[e * nm]);
      }
    });
    parallel(nglobal, nthreads, [&](long long a, long long b, int) {
      for (long long i = a; i < b; ++i) {
        double s = 0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) s += sign[col[j]] * lo[col[j]];
        gout[i] = s;
      }
    });
  };
  auto dots = [&](const double* a1, const double* b1, const double* a2, const double* b2, const double* a3,
                  const double* b3, double* res) {
    std::fill(part.begin(), part.end(), 0.0);
    parallel(nnd, nthreads, [&](long long a, long long b, int tid) {
      double s1 = 0, s2 = 0, s3 = 0;
      for (long long i = a; i < b; ++i) {
        s1 += a1[i] * b1[i];
        if (a2) s2 += a2[i] * b2[i];
        if (a3) s3 += a3[i] * b3[i];
      }
      part[3 * tid] = s1;
      part[3 * tid + 1] = s2;
      part[3 * tid + 2] = s3;
    });
    res[0] = res[1] = res[2] = 0;
    for (size_t k = 0; k < part.size() / 3; ++k)
      for (int c = 0; c < 3; ++c) res[c] += part[3 * k + c];
  };
  for (int i = 0; i < nnd; ++i) {
    r[i] = rhs[ndir + i];
    x[ndir + i] = 0.0;
  }
  double d3[3];
  dots(r.data(), r.data(), nullptr, nullptr, nullptr, nullptr, d3);
  double eps = d3[0], mag = 0;
  for (int i = 0; i < nglobal; ++i) mag += rhs[i] * rhs[i];
  mag = mag > 1e-6 ? mag : 1.0;
  tol = std::max(tol, 1e-16);
  if (eps < tol * tol * mag) {
    if (final_eps) *final_eps = eps;
    return 0;
  }
  for (int i = 0; i < nnd; ++i) wA[ndir + i] = dinv[i] * r[i];
  apply(wA, sA);
  dots(r.data(), wA.data() + ndir, sA.data() + ndir, wA.data() + ndir, nullptr, nullptr, d3);
  double rho = d3[0], mu = d3[1], beta = 0.0, alpha = rho / mu;
  int iters = 1, k = 0;
  while (true) {
    if (k >= max_iter) {
      if (final_eps) *final_eps = eps;
      return -1;
    }
    parallel(nnd, nthreads, [&](long long a, long long b, int) {
      for (long long i = a; i < b; ++i) {
        p[i] = beta * p[i] + wA[ndir + i];
        q[i] = beta * q[i] + sA[ndir + i];
        x[ndir + i] += alpha * p[i];
        r[i] -= alpha * q[i];
        wA[ndir + i] = dinv[i] * r[i];
      }
    });
    apply(wA, sA);
    dots(r.data(), wA.data() + ndir, sA.data() + ndir, wA.data() + ndir, r.data(), r.data(), d3);
    const double rho_new = d3[0];
    mu = d3[1];
    eps = d3[2];
    iters++;
    if (eps < tol * tol * mag) break;
    beta = rho_new / rho;
    alpha = rho_new / (mu - rho_new * beta / alpha);
    rho = rho_new;
    k++;
  }
  if (final_eps) *final_eps = eps;
  return iters;
}

}  // extern "C"
